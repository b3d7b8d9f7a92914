// extern "C" boundary (include/imsrg_gb300.h): model spaces, device-resident
// operators, the IMSRG(2) terms, CommutatorScalarScalar and the BCH transform.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <cstdint>
#include <cstring>
#include <exception>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/imsrg_gb300.h"
#include "capi_internal.hpp"
#include "kernels.cuh"
#include "prof.hpp"
#include "space.hpp"

using namespace imsrg;

namespace {

thread_local std::string g_err;

int fail(int code, const std::string& msg)
{
  g_err = msg;
  return code;
}

#define CUDA_TRY(expr)                                                                  \
  do {                                                                                  \
    cudaError_t _e = (expr);                                                            \
    if (_e != cudaSuccess)                                                              \
      return fail(IMSRG_ERR_CUDA, std::string(#expr) + ": " + cudaGetErrorString(_e)); \
  } while (0)

// Commutator::comm_term_on (src/Commutator.cc): the scalar terms, then the
// scalar-tensor terms CommutatorScalarTensor consults (src/Commutator.cc:
// 459-482; comm222_pp_hh_221st runs when both comm222_pp_hhst and comm221st
// are on)
enum Term {
  T110 = 0, T220, T111, T121, T122, T221, T222PPHH, T222PH, NSCALAR_TERMS,
  TS111 = NSCALAR_TERMS, TS121, TS122, TS222PPHH, TS221, TS222PH, NTERMS
};
const char* kTermNames[NTERMS] = {"comm110ss",  "comm220ss",  "comm111ss",       "comm121ss",
                                  "comm122ss",  "comm221ss",  "comm222_pp_hhss", "comm222_phss",
                                  "comm111st",  "comm121st",  "comm122st",       "comm222_pp_hhst",
                                  "comm221st",  "comm222_phst"};
std::mutex g_mu;
bool g_term_on[NTERMS] = {true, true, true, true, true, true, true, true, true, true, true, true, true, true};
int g_default_precision = IMSRG_PREC_FP64;

template <class T>
T* dmalloc(size_t count)
{
  void* p = nullptr;
  if (cudaMalloc(&p, std::max<size_t>(1, count) * sizeof(T)) != cudaSuccess) throw std::runtime_error("cudaMalloc");
  return (T*)p;
}

template <class T>
T* dcopy(const std::vector<T>& v)
{
  T* p = dmalloc<T>(v.size());
  if (!v.empty() && cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    throw std::runtime_error("cudaMemcpy");
  return p;
}

}  // namespace

namespace imsrg {
int set_error(int code, const char* msg) { return fail(code, msg); }
}  // namespace imsrg

// struct imsrg_space / imsrg_op: capi_internal.hpp


namespace {

std::vector<int> tile_pairs(const std::vector<GemmJobDev>& jobs, int tile)
{
  // jobs in decreasing size order so the big tiles start first
  std::vector<int> order(jobs.size());
  for (size_t i = 0; i < jobs.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return jobs[a].m > jobs[b].m; });
  std::vector<int> out;
  for (int j : order) {
    int nt = (jobs[j].m + tile - 1) / tile;
    for (int a = 0; a < nt; ++a)
      for (int b = a; b < nt; ++b) {
        out.push_back(j);
        out.push_back(a);
        out.push_back(b);
      }
  }
  return out;
}

GemmJobDev to_dev(const SymGemmJob& j, int bsel, int sign, int accumulate)
{
  GemmJobDev d{};
  d.a_off = j.a_off;
  d.b_off = j.b_off;
  d.out_off = j.out_off;
  d.m = j.m;
  d.K = j.K;
  d.lda = j.lda;
  d.ldb = j.ldb;
  d.ldo = j.ldo;
  d.kidx_off = j.kidx_off;
  d.w_off = j.w_off;
  d.phase_off = j.phase_off;
  d.bsel = bsel;
  d.sign = sign;
  d.accumulate = accumulate;
  d.bscale = 1.0;
  return d;
}

void setup_device_lists(imsrg_space* sp)
{
  Space& s = *sp->s;
  upload_space(s);
  sp->d_holes = sp->track(dcopy(s.holes));
  // ladder: bscale = hY (launch), sign = hZ (launch), accumulate into Z
  for (const SymGemmJob& j : s.ladder_jobs) sp->ladder_jobs.push_back(to_dev(j, 0, 0, 1));
  sp->d_ladder_jobs = sp->track(dcopy(sp->ladder_jobs));
  std::vector<int> lp = tile_pairs(sp->ladder_jobs, symgemm_fp64_tile());
  sp->n_ladder_pairs = (int)lp.size() / 3;
  sp->d_ladder_pairs = sp->track(dcopy(lp));
  // Zbar: head (B = Ybar^T, sign = hZ), tail (B = Yflip^T, sign +1, phases), overwrite
  for (size_t t = 0; t < s.zbar_jobs.size(); ++t) {
    bool tail = (t % 2) == 1;
    sp->zbar_jobs.push_back(to_dev(s.zbar_jobs[t], tail ? 1 : 0, tail ? 1 : 0, 0));
  }
  sp->d_zbar_jobs = sp->track(dcopy(sp->zbar_jobs));
  std::vector<int> zp = tile_pairs(sp->zbar_jobs, symgemm_fp64_tile());
  sp->n_zbar_pairs = (int)zp.size() / 3;
  sp->d_zbar_pairs = sp->track(dcopy(zp));
  // comm122 symmetrisation tiles (all 32x32 tiles of every block)
  std::vector<int> t122, tinv;
  for (int c = 0; c < s.nch; ++c) {
    int n = s.ch[c].n();
    int nt = (n + 31) / 32;
    for (int a = 0; a < nt; ++a)
      for (int b = 0; b < nt; ++b) {
        t122.push_back(c);
        t122.push_back(a);
        t122.push_back(b);
      }
    for (int a = 0; a < nt; ++a)
      for (int b = a; b < nt; ++b) {
        tinv.push_back(c);
        tinv.push_back(a);
        tinv.push_back(b);
      }
  }
  // Inverse-Pandya tiles ordered so that blocks running at the same time
  // cover the same orbit region for every J: a Zbar element is read by the
  // elements of one orbit quadruple in all J channels, so this turns most of
  // those rereads into L2 hits.  Key: (parity/Tz family, global index of the
  // first bra, of the first ket, J).
  {
    struct Key {
      int fam;
      int gb, gk, J;
      int t;
    };
    std::vector<Key> keys;
    for (size_t t = 0; t < tinv.size() / 3; ++t) {
      int c = tinv[3 * t], a = tinv[3 * t + 1], b = tinv[3 * t + 2];
      const Chan& C = s.ch[c];
      keys.push_back({c % 6, ket_index(s.norb, C.p[32 * a], C.q[32 * a]), ket_index(s.norb, C.p[32 * b], C.q[32 * b]),
                      C.J, (int)t});
    }
    std::stable_sort(keys.begin(), keys.end(), [](const Key& x, const Key& y) {
      if (x.fam != y.fam) return x.fam < y.fam;
      if (x.gb != y.gb) return x.gb < y.gb;
      if (x.gk != y.gk) return x.gk < y.gk;
      return x.J < y.J;
    });
    std::vector<int> sorted;
    for (const Key& k : keys)
      for (int f = 0; f < 3; ++f) sorted.push_back(tinv[3 * k.t + f]);
    tinv.swap(sorted);
  }
  for (int c = 0; c < s.nch; ++c) {
    int ncc = s.cc[c].n();
    int K = 2 * s.cc_nph[c];
    if (ncc == 0) continue;
    if (K == 0) sp->zbar_zero.push_back({s.zb_off[c], (int64_t)ncc * 2 * ncc});
  }
  sp->n_sym122 = (int)t122.size() / 3;
  sp->d_sym122 = sp->track(dcopy(t122));
  // tile pairs (a <= b) of the fused split-form comm122ss
  {
    std::vector<int> tu;
    for (int c = 0; c < s.nch; ++c) {
      int nt = (s.ch[c].n() + 31) / 32;
      for (int a = 0; a < nt; ++a)
        for (int b = a; b < nt; ++b) {
          tu.push_back(c);
          tu.push_back(a);
          tu.push_back(b);
        }
    }
    sp->n_sym122u = (int)tu.size() / 3;
    sp->d_sym122u = sp->track(dcopy(tu));
  }
  sp->n_pinv = (int)tinv.size() / 3;
  sp->d_pinv = sp->track(dcopy(tinv));
  build_invq_tasks(s, sp->invq_budget);
  sp->n_invq = (int)s.invq_tasks.size() / 4;
  sp->d_invq = sp->track(dcopy(s.invq_tasks));
  sp->d_cls_list = sp->track(dcopy(s.cls_list));
  sp->d_cls_off = sp->track(dcopy(s.cls_off));
  sp->d_cls_sort = sp->track(dcopy(s.cls_sort));
  // norm chunks: every 2b block in pieces of <= 65536 elements, weight (2J+1)^2
  std::vector<long long> no;
  std::vector<int> nl;
  std::vector<double> nw;
  for (int c = 0; c < s.nch; ++c) {
    long long nn = (long long)s.ch[c].n() * s.ch[c].n();
    double w = (double)(2 * s.ch[c].J + 1) * (2 * s.ch[c].J + 1);
    for (long long o = 0; o < nn; o += 65536) {
      no.push_back(s.ch[c].off + o);
      nl.push_back((int)std::min<long long>(65536, nn - o));
      nw.push_back(w);
    }
  }
  sp->n_norm = (int)no.size();
  sp->d_norm_off = sp->track(dcopy(no));
  sp->d_norm_len = sp->track(dcopy(nl));
  sp->d_norm_w = sp->track(dcopy(nw));
  sp->d_norm_partial = sp->track(dmalloc<double>(sp->n_norm + 1));
  sp->h_norm_partial.resize(sp->n_norm + 1);
  sp->d_status = sp->track(dmalloc<int>(16));
  cudaMemset(sp->d_status, 0, 16 * sizeof(int));
}

// ------------------------------------------------------------------ tuning
int rebuild_invq(imsrg_space* sp);
void drop_invd(imsrg_space* sp);

// Names of the tunable parameters of a space (imsrg_space_set_tuning).
const char* kTuneNames[] = {"ladder.tile",  "ladder.stages", "ladder.schedule",     "zbar.tile",
                            "zbar.stages",  "zbar.schedule", "inverse.split",       "inverse.fp64",
                            "inverse.quad_budget", "inverse.desc_stage", "inverse.desc_results",
                            "inverse.desc_weights", "inverse.desc_ilp", "comm122.fused", "ladder.digits",
                            "zbar.digits"};
constexpr int kNTune = sizeof(kTuneNames) / sizeof(kTuneNames[0]);

int* tune_slot(imsrg_space* sp, int t)
{
  switch (t) {
    case 0: return &sp->opt_ladder.tn;
    case 1: return &sp->opt_ladder.stages;
    case 2: return &sp->opt_ladder.sched;
    case 3: return &sp->opt_zbar.tn;
    case 4: return &sp->opt_zbar.stages;
    case 5: return &sp->opt_zbar.sched;
    case 6: return &sp->inv_split;
    case 7: return &sp->inv_fp64;
    case 8: return &sp->invq_budget;
    case 9: return &sp->invd_stage;
    case 10: return &sp->invd_res;
    case 11: return &sp->invd_weights;
    case 12: return &sp->invd_ilp;
    case 13: return &sp->comm122_fused;
    case 14: return &sp->opt_ladder.digits;
    case 15: return &sp->opt_zbar.digits;
  }
  return nullptr;
}

bool tune_valid(int t, int v)
{
  switch (t) {
    case 0: case 3: return v == 0 || v == 32 || v == 64;
    case 1: case 4: return v == 0 || (v >= 2 && v <= 6);
    case 2: case 5: return v == 0 || v == 1;
    case 6: return v >= 0 && v <= 2;
    case 7: return v == 0 || v == 1;
    case 8: return v >= 8192 && v <= 160 * 1024;
    case 9: return v >= 64 && v <= 8192;
    case 10: return v >= 64 && v <= (1 << 20);
    case 11: return v == 0 || v == 1;
    case 12: return v == 1 || v == 2 || v == 4;
    case 13: return v == 0 || v == 1;
    case 14: case 15: return v == 0 || (v >= 5 && v <= 7);
  }
  return false;
}

// sets parameter t; with the device tables built, the plans it shapes are
// dropped (and rebuilt on next use)
int tune_apply(imsrg_space* sp, int t, int v)
{
  if (!tune_valid(t, v)) return fail(IMSRG_ERR_ARG, std::string("bad value for ") + kTuneNames[t]);
  int* slot = tune_slot(sp, t);
  if (*slot == v) return IMSRG_OK;
  *slot = v;
  if (t == 0 || t == 3) (t == 0 ? sp->opt_ladder : sp->opt_zbar).nacc = v == 64 ? 1 : (v == 32 ? 2 : 0);
  if (!sp->dev_ready) return IMSRG_OK;
  if ((t <= 2 || t == 14) && sp->split_ladder) {
    split_plan_destroy(sp->split_ladder);
    sp->split_ladder = nullptr;
  }
  if (((t >= 3 && t <= 5) || t == 15) && sp->split_zbar) {
    split_plan_destroy(sp->split_zbar);
    sp->split_zbar = nullptr;
  }
  if (t == 8) return rebuild_invq(sp);
  if (t >= 9 && t <= 11) drop_invd(sp);
  return IMSRG_OK;
}

int tune_index(const char* name)
{
  for (int t = 0; t < kNTune; ++t)
    if (name && std::strcmp(name, kTuneNames[t]) == 0) return t;
  return -1;
}

// The tuning file: one line per tuned space, "arena=<len> norb=<n>
// name=value ...", written by imsrg_gb300.autotune.  Found at
// $IMSRG_GB300_TUNING ("off": none), else tuning/gb300.txt beside the
// library's directory (imsrg_gb300/tuning/ for the in-tree build).
std::string tuning_file_path()
{
  const char* env = std::getenv("IMSRG_GB300_TUNING");
  if (env && *env) return std::strcmp(env, "off") == 0 ? std::string() : std::string(env);
  Dl_info info;
  if (!dladdr((void*)&tuning_file_path, &info) || !info.dli_fname) return std::string();
  std::string so(info.dli_fname);
  size_t cut = so.find_last_of('/');
  std::string dir = cut == std::string::npos ? std::string(".") : so.substr(0, cut);
  return dir + "/../tuning/gb300.txt";
}

void apply_tuning_file(imsrg_space* sp)
{
  std::string path = tuning_file_path();
  if (path.empty()) return;
  std::ifstream in(path);
  if (!in) return;
  std::string line;
  int lineno = 0;
  while (std::getline(in, line)) {
    ++lineno;
    if (line.empty() || line[0] == '#') continue;
    std::istringstream ls(line);
    std::string tok;
    std::vector<std::pair<std::string, long long>> kv;
    while (ls >> tok) {
      size_t eq = tok.find('=');
      if (eq == std::string::npos) continue;
      kv.push_back({tok.substr(0, eq), std::atoll(tok.c_str() + eq + 1)});
    }
    long long arena = -1, norb = -1;
    for (auto& p : kv) {
      if (p.first == "arena") arena = p.second;
      if (p.first == "norb") norb = p.second;
    }
    if (arena != sp->s->arena || norb != sp->s->norb) continue;
    for (auto& p : kv) {
      int t = tune_index(p.first.c_str());
      if (t >= 0 && tune_valid(t, (int)p.second)) tune_apply(sp, t, (int)p.second);
    }
    sp->tuning_source = path + ":" + std::to_string(lineno);
    return;
  }
}

// device tables are built on first device use, so a space can be created and
// queried on a machine without a GPU
int ensure_device(imsrg_space* sp)
{
  std::lock_guard<std::mutex> g(sp->mu);
  if (sp->dev_ready) return IMSRG_OK;
  int dev = -1;
  CUDA_TRY(cudaGetDevice(&dev));
  apply_tuning_file(sp);
  try {
    setup_device_lists(sp);
  } catch (std::exception& e) {
    return fail(IMSRG_ERR_CUDA, std::string("device tables: ") + e.what());
  }
  sp->device = dev;
  int rc = noalloc_setup(sp, dev);
  if (rc) return rc;
  sp->dev_ready = true;
  return IMSRG_OK;
}

// lazily allocated scratch of a space
int ensure_scratch(imsrg_space* sp, bool pandya, bool w2)
{
  try {
    Space& s = *sp->s;
    if (pandya && !sp->d_zb) {
      sp->d_xb = sp->track(dmalloc<double>(s.xb_total));
      sp->d_yt = sp->track(dmalloc<double>(s.xb_total));
      sp->d_yf = sp->track(dmalloc<double>(s.xb_total));
      sp->d_zb = sp->track(dmalloc<double>(s.zb_total));
    }
    if (w2 && !sp->d_w2) sp->d_w2 = sp->track(dmalloc<double>(s.arena));
  } catch (std::exception& e) {
    return fail(IMSRG_ERR_NOMEM, std::string("scratch allocation failed: ") + e.what());
  }
  return IMSRG_OK;
}

// untracks and frees one device allocation of the space
void drop_alloc(imsrg_space* sp, void* p)
{
  if (!p) return;
  auto it = std::find(sp->allocs.begin(), sp->allocs.end(), p);
  if (it != sp->allocs.end()) sp->allocs.erase(it);
  cudaFree(p);
}

// the quadruple blocks of the split form's inverse Pandya transform, rebuilt
// for the space's shared-memory budget
int rebuild_invq(imsrg_space* sp)
{
  Space& s = *sp->s;
  drop_alloc(sp, sp->d_invq);
  drop_alloc(sp, sp->d_cls_list);
  drop_alloc(sp, sp->d_cls_off);
  drop_alloc(sp, sp->d_cls_sort);
  sp->d_invq = nullptr;
  sp->d_cls_list = sp->d_cls_off = nullptr;
  sp->d_cls_sort = nullptr;
  try {
    build_invq_tasks(s, sp->invq_budget);
    sp->n_invq = (int)s.invq_tasks.size() / 4;
    sp->d_invq = sp->track(dcopy(s.invq_tasks));
    sp->d_cls_list = sp->track(dcopy(s.cls_list));
    sp->d_cls_off = sp->track(dcopy(s.cls_off));
    sp->d_cls_sort = sp->track(dcopy(s.cls_sort));
  } catch (std::exception& e) {
    sp->n_invq = 0;
    return fail(IMSRG_ERR_NOMEM, std::string("inverse Pandya blocks: ") + e.what());
  }
  return IMSRG_OK;
}

void drop_invd(imsrg_space* sp)
{
  for (void* p : sp->invd_allocs) cudaFree(p);
  sp->invd_allocs.clear();
  sp->invd = InvdDev{};
  sp->invd_ready = false;
}

// the inverse Pandya descriptors of the space (built on first use)
int ensure_invd(imsrg_space* sp)
{
  if (sp->invd_ready) return IMSRG_OK;
  drop_invd(sp);
  try {
    InvdPlan plan;
    build_invd(*sp->s, plan, sp->invd_stage, sp->invd_res, sp->invd_weights != 0);
    auto up = [&](const auto& v) {
      auto* p = dcopy(v);
      sp->invd_allocs.push_back((void*)p);
      return p;
    };
    sp->invd.blocks = up(plan.blocks);
    sp->invd.wblk = up(plan.wblk);
    sp->invd.wrow = up(plan.wrow);
    sp->invd.sslot = up(plan.sslot);
    sp->invd.sidx = up(plan.sidx);
    sp->invd.dA = up(plan.dA);
    sp->invd.dB = up(plan.dB);
    sp->invd.nblocks = (int)plan.blocks.size();
    long long upper = 0;  // upper-triangle elements (diagonal included) of every two-body block
    for (const Chan& C : sp->s->ch) upper += (long long)C.n() * (C.n() + 1) / 2;
    sp->invd.covers_all = (long long)plan.dA.size() == upper;
    sp->invd.stage_max = plan.stage_max;
    sp->invd.staged_weights = sp->invd_weights != 0;
  } catch (std::exception& e) {
    drop_invd(sp);
    return fail(IMSRG_ERR_NOMEM, std::string("inverse Pandya descriptors: ") + e.what());
  }
  sp->invd_ready = true;
  return IMSRG_OK;
}

// AddInversePandyaTransformation of zb into Z with the kernel the space's
// tuning selects for the form (grouped: nz pairs at the offsets zo)
int inverse_pandya(imsrg_space* sp, const double* zb, double* Z, int hZ, int prec, cudaStream_t st,
                   const long long* zo = nullptr, int nz = 1, const void* w2 = nullptr, int w2mode = 0)
{
  Space& s = *sp->s;
  const int variant = prec == IMSRG_PREC_SPLIT ? sp->inv_split : (sp->inv_fp64 ? 2 : 0);
  if (variant == 1 || variant == 2) {
    int rc = ensure_invd(sp);
    if (rc) return rc;
    sp->invd.ilp = sp->invd_ilp;
    CUDA_TRY(launch_pandya_inv_desc(s, sp->invd, variant == 1, zb, Z, hZ, st, zo, nz, w2, w2mode));
    return IMSRG_OK;
  }
  if (w2mode) return fail(IMSRG_ERR_ARG, "comm122ss's update folds only into the descriptor inverse kernel");
  if (prec == IMSRG_PREC_SPLIT && sp->n_invq > 0) {
    CUDA_TRY(launch_pandya_inv_ff(s, zb, Z, hZ, sp->d_invq, sp->n_invq, sp->d_cls_list, sp->d_cls_off, sp->d_cls_sort,
                                  s.invq_smem, st, zo, nz));
    return IMSRG_OK;
  }
  if (zo) return fail(IMSRG_ERR_UNSUPPORTED, "grouped inverse Pandya needs the quadruple or descriptor kernel");
  CUDA_TRY(launch_pandya_inv(s, zb, Z, hZ, sp->d_pinv, sp->n_pinv, st));
  return IMSRG_OK;
}

int check_ops(const imsrg_op* X, const imsrg_op* Y, const imsrg_op* Z)
{
  if (!X || !Y || !Z) return fail(IMSRG_ERR_ARG, "null operator");
  if (X->tl || Y->tl || Z->tl)
    return fail(IMSRG_ERR_UNSUPPORTED, "tensor operator passed to a scalar-scalar term (use imsrg_commutator_scalar_tensor)");
  if (X->sp != Y->sp || X->sp != Z->sp) return fail(IMSRG_ERR_ARG, "operators belong to different model spaces");
  if ((X->herm != 1 && X->herm != -1) || (Y->herm != 1 && Y->herm != -1))
    return fail(IMSRG_ERR_UNSUPPORTED, "X and Y must be hermitian or anti-hermitian");
  if (Z->herm != 1 && Z->herm != -1) return fail(IMSRG_ERR_UNSUPPORTED, "Z must be hermitian or anti-hermitian");
  return IMSRG_OK;
}

cudaStream_t S_(void* st) { return (cudaStream_t)st; }

// ---------------------------------------------------------------- the terms
int do_111_110(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, bool do111, bool do110, cudaStream_t st)
{
  // comm110ss returns early when X and Y have the same hermiticity (src/Commutator.cc:567-570)
  if (do110 && X->herm == Y->herm) do110 = false;
  if (!do111 && !do110) return IMSRG_OK;
  ProfScope ps(do111 ? (do110 ? "comm111ss+comm110ss" : "comm111ss") : "comm110ss", st);
  CUDA_TRY(launch_comm111_110(*X->sp->s, X->d, Y->d, Z->d, do111, do110, st));
  return IMSRG_OK;
}

int do_220(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  if (X->herm == Y->herm) return IMSRG_OK;  // src/Commutator.cc:606-609
  ProfScope ps("comm220ss", st);
  CUDA_TRY(launch_comm220(*X->sp->s, X->d, Y->d, Z->d, X->herm, st));
  return IMSRG_OK;
}

int do_121(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st)
{
  ProfScope ps("comm121ss", st);
  CUDA_TRY(launch_comm121(*X->sp->s, X->sp->d_holes, X->d, Y->d, Z->d, Z->herm, st));
  return IMSRG_OK;
}

// Split form, first half: the (hi, lo) float-pair copies of X and Y
int prep_122_df(const imsrg_op* X, const imsrg_op* Y, cudaStream_t st)
{
  imsrg_space* sp = X->sp;
  int rc = ensure_scratch(sp, false, true);
  if (rc) return rc;
  try {
    if (!sp->d_xf) sp->d_xf = sp->track(dmalloc<float2>(sp->s->arena));
    if (!sp->d_yff) sp->d_yff = sp->track(dmalloc<float2>(sp->s->arena));
  } catch (std::exception&) {
    return fail(IMSRG_ERR_NOMEM, "comm122ss double-float scratch");
  }
  ProfScope ps("comm122ss prep", st);
  CUDA_TRY(launch_to_ff(*sp->s, X->d, sp->d_xf, st));
  CUDA_TRY(launch_to_ff(*sp->s, Y->d, sp->d_yff, st));
  return IMSRG_OK;
}

// FP64 form: FP64 gathers (the plain form keeps every term in FP64).
// Split form: the same gathers in double-float on the FP32 pipe (prepared:
// the float-pair copies are already made, on a stream ordered before st).
// fold_sym: only W2 here; the inverse Pandya kernel applies Z -= W2 + hZ W2^T
int do_122(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st, int prec = IMSRG_PREC_FP64,
           bool prepared = false, bool fold_sym = false)
{
  imsrg_space* sp = X->sp;
  int rc = ensure_scratch(sp, false, true);
  if (rc) return rc;
  if (prec == IMSRG_PREC_SPLIT) {
    if (!prepared && (rc = prep_122_df(X, Y, st))) return rc;
    ProfScope ps("comm122ss", st);
    if (sp->comm122_fused)
      CUDA_TRY(launch_comm122_fused_df(*sp->s, X->d, Y->d, Z->d, sp->d_xf, sp->d_yff, Z->herm, sp->d_sym122u,
                                       sp->n_sym122u, st));
    else
      CUDA_TRY(launch_comm122_df(*sp->s, X->d, Y->d, Z->d, sp->d_xf, sp->d_yff, (float2*)sp->d_w2, Z->herm,
                                 sp->d_sym122, sp->n_sym122, st, nullptr, 1, !fold_sym));
    return IMSRG_OK;
  }
  ProfScope ps("comm122ss", st);
  CUDA_TRY(launch_comm122(*sp->s, X->d, Y->d, Z->d, sp->d_w2, Z->herm, sp->d_sym122, sp->n_sym122, st, nullptr, 1,
                          !fold_sym));
  return IMSRG_OK;
}

// Mz: the two-body blocks of Mpp - Mhh when already available (the ladder
// product accumulated onto a zeroed Z), else nullptr (dot products)
int do_221_1b(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, cudaStream_t st, const double* Mz = nullptr)
{
  ProfScope ps("comm221ss", st);
  CUDA_TRY(launch_comm221_1b(*X->sp->s, X->d, Y->d, Z->d, X->herm, Z->herm, Mz, st));
  return IMSRG_OK;
}

int check_status(imsrg_space* sp, cudaStream_t st)
{
  int h = 0;
  CUDA_TRY(cudaMemcpyAsync(&h, sp->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  if (h != 0) {
    cudaMemsetAsync(sp->d_status, 0, sizeof(int), st);
    return fail(IMSRG_ERR_KERNEL, "a kernel reported error status " + std::to_string(h));
  }
  return IMSRG_OK;
}

int ensure_split(imsrg_space* sp)
{
  try {
    if (!sp->split_ladder) sp->split_ladder = split_plan_create(*sp->s, sp->ladder_jobs, 0, sp->opt_ladder);
    if (!sp->split_zbar) sp->split_zbar = split_plan_create(*sp->s, sp->zbar_jobs, 1, sp->opt_zbar);
  } catch (std::exception& e) {
    return fail(IMSRG_ERR_NOMEM, std::string("split-precision plan: ") + e.what());
  }
  return IMSRG_OK;
}

// overwrite: Z2 is known to be zero (fresh commutator), so the split product
// writes its blocks instead of read-modify-write
int do_ladder(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int prec, cudaStream_t st, bool overwrite = false)
{
  imsrg_space* sp = X->sp;
  Space& s = *sp->s;
  ProfScope ps("comm222_pp_hhss", st);
  if (prec == IMSRG_PREC_SPLIT) {
    int rc = ensure_split(sp);
    if (rc) return rc;
    split_plan_set_accumulate(sp->split_ladder, overwrite ? 0 : -1);
    CUDA_TRY(launch_symgemm_split(sp->split_ladder, X->d, Y->d, Y->d, Z->d, s.work.kidx, s.work.kweight,
                                  s.work.phase_tab, sp->d_status, Z->herm, (double)Y->herm, st));
    return IMSRG_OK;
  }
  if (prec != IMSRG_PREC_FP64) return fail(IMSRG_ERR_ARG, "unknown precision");
  CUDA_TRY(launch_symgemm_fp64(sp->d_ladder_jobs, sp->d_ladder_pairs, sp->n_ladder_pairs, X->d, Y->d, Y->d, Z->d,
                               s.work.kidx, s.work.kweight, s.work.phase_tab, Z->herm, (double)Y->herm, st));
  return IMSRG_OK;
}

// comm222_phss, first half: the Pandya-transformed operands (X bar, Y bar,
// Y bar flipped) and the zero blocks of Z bar
int prep_ph(const imsrg_op* X, const imsrg_op* Y, int prec, cudaStream_t st)
{
  imsrg_space* sp = X->sp;
  Space& s = *sp->s;
  int rc = ensure_scratch(sp, true, false);
  if (rc) return rc;
  ProfScope ps("Pandya transform of X, Y", st);
  CUDA_TRY(launch_pandya_fwd(s, X->d, Y->d, Y->herm, sp->d_xb, sp->d_yt, sp->d_yf, prec == IMSRG_PREC_SPLIT, st));
  for (auto& zr : sp->zbar_zero) CUDA_TRY(cudaMemsetAsync(sp->d_zb + zr.first, 0, zr.second * sizeof(double), st));
  return IMSRG_OK;
}

// prepared: prep_ph already ran, on a stream ordered before st
// fold_w2: also apply comm122ss's Z -= W2 + hZ W2^T (W2 already computed on st)
int do_ph(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int prec, cudaStream_t st, bool prepared = false,
          bool fold_w2 = false)
{
  imsrg_space* sp = X->sp;
  Space& s = *sp->s;
  int rc = ensure_scratch(sp, true, false);
  if (rc) return rc;
  if (!prepared && (rc = prep_ph(X, Y, prec, st))) return rc;
  ProfScope ps("comm222_phss", st);
  int slot = prof_begin("Build Z_bar", st);
  if (prec == IMSRG_PREC_SPLIT) {
    rc = ensure_split(sp);
    if (rc) return rc;
    // the descriptor inverse kernels read only Zbar's upper triangle
    split_plan_set_mirror(sp->split_zbar, sp->inv_split == 0 ? 1 : 0);
    CUDA_TRY(launch_symgemm_split(sp->split_zbar, sp->d_xb, sp->d_yt, sp->d_yf, sp->d_zb, s.work.kidx,
                                  s.work.kweight, s.work.phase_tab, sp->d_status, Z->herm, 1.0, st));
  } else if (prec == IMSRG_PREC_FP64) {
    CUDA_TRY(launch_symgemm_fp64(sp->d_zbar_jobs, sp->d_zbar_pairs, sp->n_zbar_pairs, sp->d_xb, sp->d_yt, sp->d_yf,
                                 sp->d_zb, s.work.kidx, s.work.kweight, s.work.phase_tab, Z->herm, 1.0, st));
  } else {
    return fail(IMSRG_ERR_ARG, "unknown precision");
  }
  prof_end(slot, st);
  ProfScope pinv("InversePandyaTransformation", st);
  return inverse_pandya(sp, sp->d_zb, Z->d, Z->herm, prec, st, nullptr, 1, fold_w2 ? (const void*)sp->d_w2 : nullptr,
                        fold_w2 ? (prec == IMSRG_PREC_SPLIT ? 1 : 2) : 0);
}

int z_herm(int hx, int hy) { return (hx == hy) ? -1 : 1; }

int commutator_impl(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int prec, cudaStream_t st)
{
  if (!X || !Y || !Z) return fail(IMSRG_ERR_ARG, "null operator");
  if (Z == X || Z == Y) return fail(IMSRG_ERR_ARG, "Z must not alias X or Y");
  Z->herm = z_herm(X->herm, Y->herm);
  int rc = check_ops(X, Y, Z);
  if (rc) return rc;
  bool on[NTERMS];
  {
    std::lock_guard<std::mutex> g(g_mu);
    std::copy(g_term_on, g_term_on + NTERMS, on);
  }
  imsrg_space* sp = X->sp;
  if (!sp->side) {
    CUDA_TRY(cudaStreamCreateWithFlags(&sp->side, cudaStreamNonBlocking));
    CUDA_TRY(cudaEventCreateWithFlags(&sp->ev_fork, cudaEventDisableTiming));
    CUDA_TRY(cudaEventCreateWithFlags(&sp->ev_join, cudaEventDisableTiming));
  }
  cudaStream_t sd = sp->side;
  ProfScope ps("CommutatorScalarScalar", st);
  CUDA_TRY(cudaMemsetAsync(Z->d, 0, sp->s->arena * sizeof(double), st));
  // The terms add into Z in an order of our own (the sum is the same up to
  // rounding): the ladder product goes first, onto the zeroed two-body blocks,
  // so the one-body part of comm221ss can read Mpp - Mhh straight from Z2
  // instead of recomputing the pp dot products (ConstructScalarMpp_Mhh is
  // shared the same way by the reference's comm222_pp_hh_221ss).
  //
  // While the ladder product runs on st, a second stream does what does not
  // depend on it: the operand preparation of comm122ss and comm222_phss and
  // the zero- and one-body terms 111/110, 220, 121 (they write only Z0 and Z1,
  // the ladder only Z2).  The streams join before comm221ss, which reads Z2
  // and writes Z1.
  CUDA_TRY(cudaEventRecord(sp->ev_fork, st));
  CUDA_TRY(cudaStreamWaitEvent(sd, sp->ev_fork, 0));
  const bool split = prec == IMSRG_PREC_SPLIT;
  if (on[T122] && split && (rc = prep_122_df(X, Y, sd))) return rc;
  if (on[T222PH] && (rc = prep_ph(X, Y, prec, sd))) return rc;
  if ((rc = do_111_110(X, Y, Z, on[T111], on[T110], sd))) return rc;
  if (on[T220] && (rc = do_220(X, Y, Z, sd))) return rc;
  if (on[T121] && (rc = do_121(X, Y, Z, sd))) return rc;
  CUDA_TRY(cudaEventRecord(sp->ev_join, sd));
  bool ladder_first = on[T222PPHH];
  if (ladder_first && (rc = do_ladder(X, Y, Z, prec, st, true))) return rc;
  CUDA_TRY(cudaStreamWaitEvent(st, sp->ev_join, 0));
  if (on[T221] && (rc = do_221_1b(X, Y, Z, st, ladder_first ? Z->d : nullptr))) return rc;
  // comm122ss's final Z -= W2 + hZ W2^T rides in the inverse Pandya kernel,
  // which reads and writes every upper-triangle element of Z and its mirror
  // anyway, when that kernel is the descriptor one and lists every element
  bool fold = false;
  if (on[T122] && on[T222PH] && !(split && sp->comm122_fused)) {
    const int variant = split ? sp->inv_split : (sp->inv_fp64 ? 2 : 0);
    if (variant == 1 || variant == 2) {
      if ((rc = ensure_invd(sp))) return rc;
      fold = sp->invd.covers_all;
    }
  }
  if (on[T122] && (rc = do_122(X, Y, Z, st, prec, split, fold))) return rc;
  if (on[T222PH] && (rc = do_ph(X, Y, Z, prec, st, true, fold))) return rc;
  return IMSRG_OK;
}

int norm_impl(const imsrg_op* op, double* out, cudaStream_t st)
{
  imsrg_space* sp = op->sp;
  CUDA_TRY(launch_norm(*sp->s, op->d, sp->d_norm_off, sp->d_norm_len, sp->d_norm_w, sp->n_norm, sp->d_norm_partial,
                       st));
  CUDA_TRY(cudaMemcpyAsync(sp->h_norm_partial.data(), sp->d_norm_partial, (sp->n_norm + 1) * sizeof(double),
                           cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  double n2 = 0.0;
  for (int i = 0; i < sp->n_norm; ++i) n2 += sp->h_norm_partial[i];
  *out = std::sqrt(sp->h_norm_partial[sp->n_norm] + n2);
  return IMSRG_OK;
}

// splitmix64 -> uniform [-1, 1)
struct Rng {
  uint64_t s;
  uint64_t next()
  {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  double uniform() { return (double)(next() >> 11) * (2.0 / 9007199254740992.0) - 1.0; }
};

}  // namespace

// ======================================================================= ABI
extern "C" {

const char* imsrg_last_error(void) { return g_err.c_str(); }

int imsrg_space_create(int emax, int norb, const int* n, const int* l, const int* j2, const int* tz2,
                       const double* occ, imsrg_space** out)
{
  if (!out || norb <= 0 || !n || !l || !j2 || !tz2 || !occ || emax < 0) return fail(IMSRG_ERR_ARG, "bad arguments");
  *out = nullptr;
  imsrg_space* sp = new imsrg_space();
  try {
    sp->s = build_space(emax, std::vector<int>(n, n + norb), std::vector<int>(l, l + norb),
                        std::vector<int>(j2, j2 + norb), std::vector<int>(tz2, tz2 + norb),
                        std::vector<double>(occ, occ + norb));
  } catch (std::exception& e) {
    delete sp;
    return fail(IMSRG_ERR_ARG, std::string("model space: ") + e.what());
  }
  *out = sp;
  return IMSRG_OK;
}

int imsrg_space_create_reference(int emax, int A, int Z, imsrg_space** out)
{
  if (emax < 0 || A < 0 || Z < 0 || Z > A) return fail(IMSRG_ERR_ARG, "bad emax / A / Z");
  std::vector<int> n, l, j2, tz2;
  std::vector<double> occ;
  try {
    reference_orbits(emax, A, Z, n, l, j2, tz2, occ);
  } catch (std::exception& e) {
    return fail(IMSRG_ERR_ARG, e.what());
  }
  return imsrg_space_create(emax, (int)n.size(), n.data(), l.data(), j2.data(), tz2.data(), occ.data(), out);
}

void imsrg_space_destroy(imsrg_space* s) { delete s; }

int imsrg_space_sizes(const imsrg_space* sp, int* norb, int* nch, long long* arena_len)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "null space");
  if (norb) *norb = sp->s->norb;
  if (nch) *nch = sp->s->nch;
  if (arena_len) *arena_len = sp->s->arena;
  return IMSRG_OK;
}

int imsrg_space_orbit(const imsrg_space* sp, int i, int* n, int* l, int* j2, int* tz2, double* occ)
{
  if (!sp || i < 0 || i >= sp->s->norb) return fail(IMSRG_ERR_ARG, "bad orbit index");
  const Space& s = *sp->s;
  if (n) *n = s.n[i];
  if (l) *l = s.l[i];
  if (j2) *j2 = s.j2[i];
  if (tz2) *tz2 = s.tz2[i];
  if (occ) *occ = s.occ[i];
  return IMSRG_OK;
}

int imsrg_space_channel(const imsrg_space* sp, int ch, int* J, int* parity, int* Tz, int* nkets, long long* offset)
{
  if (!sp || ch < 0 || ch >= sp->s->nch) return fail(IMSRG_ERR_ARG, "bad channel index");
  const Chan& C = sp->s->ch[ch];
  if (J) *J = C.J;
  if (parity) *parity = C.parity;
  if (Tz) *Tz = C.Tz;
  if (nkets) *nkets = C.n();
  if (offset) *offset = C.off;
  return IMSRG_OK;
}

int imsrg_space_channel_kets(const imsrg_space* sp, int ch, int* p, int* q)
{
  if (!sp || ch < 0 || ch >= sp->s->nch || !p || !q) return fail(IMSRG_ERR_ARG, "bad arguments");
  const Chan& C = sp->s->ch[ch];
  std::copy(C.p.begin(), C.p.end(), p);
  std::copy(C.q.begin(), C.q.end(), q);
  return IMSRG_OK;
}

int imsrg_space_cc_channel(const imsrg_space* sp, int ch, int* J, int* parity, int* Tz, int* nkets, int* p, int* q)
{
  if (!sp || ch < 0 || ch >= sp->s->nch) return fail(IMSRG_ERR_ARG, "bad channel index");
  const Chan& C = sp->s->cc[ch];
  if (J) *J = C.J;
  if (parity) *parity = C.parity;
  if (Tz) *Tz = C.Tz;
  if (nkets) *nkets = C.n();
  if (p) std::copy(C.p.begin(), C.p.end(), p);
  if (q) std::copy(C.q.begin(), C.q.end(), q);
  return IMSRG_OK;
}

int imsrg_space_sixj(const imsrg_space* sp, int jj1, int jj2, int j3, int jj4, int jj5, int j6, double* out)
{
  if (!sp || !out) return fail(IMSRG_ERR_ARG, "bad arguments");
  *out = sixj_lookup(*sp->s, jj1, jj2, j3, jj4, jj5, j6);
  return IMSRG_OK;
}

int imsrg_space_pandya_layout(const imsrg_space* sp, int ch_cc, int* rows, int* cols, long long* offset,
                              long long* total)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "bad arguments");
  const Space& s = *sp->s;
  if (total) *total = std::max<int64_t>(1, s.xb_total);
  if (ch_cc < 0) return IMSRG_OK;
  if (ch_cc >= s.nch) return fail(IMSRG_ERR_ARG, "channel index out of range");
  if (rows) *rows = 2 * s.cc_nph[ch_cc];
  if (cols) *cols = s.cc[ch_cc].n();
  if (offset) *offset = s.xb_off[ch_cc];
  return IMSRG_OK;
}

int imsrg_pandya_transform(const imsrg_op* Z, int transpose, double* out, void* stream)
{
  if (!Z || !out) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (Z->herm != 1 && Z->herm != -1) return fail(IMSRG_ERR_UNSUPPORTED, "Z must be hermitian or anti-hermitian");
  ProfScope ps("DoPandyaTransformation", S_(stream));
  CUDA_TRY(launch_pandya_single(*Z->sp->s, Z->d, Z->herm, transpose ? 1 : 0, out, S_(stream)));
  return IMSRG_OK;
}

int imsrg_op_create(imsrg_space* sp, int hermiticity, imsrg_op** out)
{
  if (!sp || !out) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (hermiticity != 1 && hermiticity != -1) return fail(IMSRG_ERR_UNSUPPORTED, "hermiticity must be +1 or -1");
  *out = nullptr;
  int rc = ensure_device(sp);
  if (rc) return rc;
  imsrg_op* op = new imsrg_op();
  op->sp = sp;
  op->herm = hermiticity;
  op->len = sp->s->arena;
  if (cudaMalloc(&op->d, sp->s->arena * sizeof(double)) != cudaSuccess) {
    delete op;
    cudaGetLastError();
    return fail(IMSRG_ERR_NOMEM, "operator arena allocation failed");
  }
  if (cudaMemset(op->d, 0, sp->s->arena * sizeof(double)) != cudaSuccess) {
    cudaFree(op->d);
    delete op;
    return fail(IMSRG_ERR_CUDA, "operator arena memset failed");
  }
  *out = op;
  return IMSRG_OK;
}

int imsrg_op_create_tensor(imsrg_space* sp, int lam, int trank, int parity, int hermiticity, imsrg_op** out)
{
  if (!sp || !out) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (lam < 0 || trank < 0 || trank > 1 || (parity != 0 && parity != 1) || lam >= sp->s->NJ)
    return fail(IMSRG_ERR_ARG, "bad tensor rank");
  if (hermiticity != 1 && hermiticity != -1) return fail(IMSRG_ERR_UNSUPPORTED, "hermiticity must be +1 or -1");
  *out = nullptr;
  int rc = ensure_device(sp);
  if (rc) return rc;
  TensorLayout* tl = nullptr;
  try {
    std::lock_guard<std::mutex> g(sp->mu);
    tl = tensor_layout(*sp->s, lam, trank, parity);
    tensor_upload(*tl);
  } catch (std::exception& e) {
    return fail(IMSRG_ERR_NOMEM, std::string("tensor tables: ") + e.what());
  }
  imsrg_op* op = new imsrg_op();
  op->sp = sp;
  op->herm = hermiticity;
  op->tl = tl;
  op->len = tl->total;
  if (cudaMalloc(&op->d, op->len * sizeof(double)) != cudaSuccess) {
    delete op;
    cudaGetLastError();
    return fail(IMSRG_ERR_NOMEM, "operator arena allocation failed");
  }
  if (cudaMemset(op->d, 0, op->len * sizeof(double)) != cudaSuccess) {
    cudaFree(op->d);
    delete op;
    return fail(IMSRG_ERR_CUDA, "operator arena memset failed");
  }
  *out = op;
  return IMSRG_OK;
}

int imsrg_op_rank(const imsrg_op* op, int* lam, int* trank, int* parity, long long* len)
{
  if (!op) return fail(IMSRG_ERR_ARG, "null operator");
  if (lam) *lam = op->tl ? op->tl->lam : 0;
  if (trank) *trank = op->tl ? op->tl->trank : 0;
  if (parity) *parity = op->tl ? op->tl->parity : 0;
  if (len) *len = op->len;
  return IMSRG_OK;
}

int imsrg_space_tensor_layout(imsrg_space* sp, int lam, int trank, int parity, int block, int* ch_bra, int* ch_ket,
                              long long* offset, int* nblocks, long long* total)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (lam < 0 || trank < 0 || trank > 1 || (parity != 0 && parity != 1) || lam >= sp->s->NJ)
    return fail(IMSRG_ERR_ARG, "bad tensor rank");
  TensorLayout* tl = nullptr;
  {
    std::lock_guard<std::mutex> g(sp->mu);
    tl = tensor_layout(*sp->s, lam, trank, parity);
  }
  if (nblocks) *nblocks = (int)tl->bra.size();
  if (total) *total = tl->total;
  if (block < 0) return IMSRG_OK;
  if (block >= (int)tl->bra.size()) return fail(IMSRG_ERR_ARG, "block index out of range");
  if (ch_bra) *ch_bra = tl->bra[block];
  if (ch_ket) *ch_ket = tl->ket[block];
  if (offset) *offset = tl->off[block];
  return IMSRG_OK;
}

int imsrg_space_wait_selftest(imsrg_space* sp, unsigned limit, long long* cycles, unsigned* production_limit,
                              void* stream)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "null space");
  if (production_limit) *production_limit = wait_limit();
  if (limit == 0 || limit > wait_limit()) return fail(IMSRG_ERR_ARG, "limit must be in [1, the production bound]");
  cudaStream_t st = (cudaStream_t)stream;
  long long* d_cyc = nullptr;
  CUDA_TRY(cudaMalloc((void**)&d_cyc, sizeof(long long)));
  long long h = 0;
  cudaError_t e = cudaMemsetAsync(d_cyc, 0, sizeof(long long), st);
  if (e == cudaSuccess) e = launch_wait_selftest(sp->d_status, limit, d_cyc, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d_cyc, sizeof(long long), cudaMemcpyDeviceToHost, st);
  int rc = e == cudaSuccess ? check_status(sp, st) : fail(IMSRG_ERR_CUDA, cudaGetErrorString(e));
  cudaStreamSynchronize(st);
  cudaFree(d_cyc);
  if (cycles) *cycles = h;
  return rc;
}

int imsrg_space_ninej(imsrg_space* sp, int lam, int ja, int jd, int J1, int jb, int jc, int J2, int Jbra, int Jket,
                      double* out)
{
  if (!sp || !out) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (lam < 0 || lam >= sp->s->NJ) return fail(IMSRG_ERR_ARG, "bad rank");
  TensorLayout* tl = nullptr;
  {
    std::lock_guard<std::mutex> g(sp->mu);
    tl = tensor_layout(*sp->s, lam, 0, 0);
  }
  // the tabulated value the kernels read (ninej_tensor fills the table)
  DevTensor h = tensor_host_view(*tl);
  *out = ninej_get(h, ja, jb, jc, jd, J1, J2, Jbra, Jket);
  return IMSRG_OK;
}

void imsrg_op_destroy(imsrg_op* op)
{
  if (!op) return;
  cudaFree(op->d);
  delete op;
}

int imsrg_op_hermiticity(const imsrg_op* op, int* h)
{
  if (!op || !h) return fail(IMSRG_ERR_ARG, "bad arguments");
  *h = op->herm;
  return IMSRG_OK;
}

int imsrg_op_set_hermiticity(imsrg_op* op, int h)
{
  if (!op) return fail(IMSRG_ERR_ARG, "null operator");
  if (h != 1 && h != -1) return fail(IMSRG_ERR_UNSUPPORTED, "hermiticity must be +1 or -1");
  op->herm = h;
  return IMSRG_OK;
}

int imsrg_op_upload(imsrg_op* op, const double* host, void* stream)
{
  if (!op || !host) return fail(IMSRG_ERR_ARG, "bad arguments");
  CUDA_TRY(cudaMemcpyAsync(op->d, host, op->len * sizeof(double), cudaMemcpyHostToDevice, S_(stream)));
  return IMSRG_OK;
}

int imsrg_op_download(const imsrg_op* op, double* host, void* stream)
{
  if (!op || !host) return fail(IMSRG_ERR_ARG, "bad arguments");
  CUDA_TRY(cudaMemcpyAsync(host, op->d, op->len * sizeof(double), cudaMemcpyDeviceToHost, S_(stream)));
  CUDA_TRY(cudaStreamSynchronize(S_(stream)));
  return IMSRG_OK;
}

int imsrg_op_device_arena(const imsrg_op* op, double** dptr)
{
  if (!op || !dptr) return fail(IMSRG_ERR_ARG, "bad arguments");
  *dptr = op->d;
  return IMSRG_OK;
}

int imsrg_op_zero(imsrg_op* op, void* stream)
{
  if (!op) return fail(IMSRG_ERR_ARG, "null operator");
  CUDA_TRY(cudaMemsetAsync(op->d, 0, op->len * sizeof(double), S_(stream)));
  return IMSRG_OK;
}

int imsrg_op_copy(imsrg_op* dst, const imsrg_op* src, void* stream)
{
  if (!dst || !src || dst->sp != src->sp) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (dst->tl != src->tl) return fail(IMSRG_ERR_ARG, "operators of different tensor rank");
  if (dst == src) return IMSRG_OK;
  CUDA_TRY(cudaMemcpyAsync(dst->d, src->d, src->len * sizeof(double), cudaMemcpyDeviceToDevice, S_(stream)));
  dst->herm = src->herm;
  return IMSRG_OK;
}

int imsrg_op_scale(imsrg_op* op, double a, void* stream)
{
  if (!op) return fail(IMSRG_ERR_ARG, "null operator");
  CUDA_TRY(launch_scale(op->d, a, op->len, S_(stream)));
  return IMSRG_OK;
}

int imsrg_op_axpy(imsrg_op* y, double a, const imsrg_op* x, void* stream)
{
  if (!y || !x || y->sp != x->sp) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (y->tl != x->tl) return fail(IMSRG_ERR_ARG, "operators of different tensor rank");
  CUDA_TRY(launch_axpy(y->d, x->d, a, y->len, S_(stream)));
  return IMSRG_OK;
}

int imsrg_op_norm(const imsrg_op* op, double* out, void* stream)
{
  if (!op || !out) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (op->tl) return tensor_norm_dev(op, out, S_(stream));
  return norm_impl(op, out, S_(stream));
}

int imsrg_op_fill_random(imsrg_op* op, unsigned long long seed, void* stream)
{
  if (!op) return fail(IMSRG_ERR_ARG, "null operator");
  if (op->tl) return fail(IMSRG_ERR_UNSUPPORTED, "random fill of a tensor operator is not on the GPU path");
  const Space& s = *op->sp->s;
  std::vector<double> a((size_t)s.arena, 0.0);
  Rng rng{seed * 0x2545F4914F6CDD1Dull + 0x1234567ull};
  double sg = op->herm == 1 ? 1.0 : -1.0;
  a[0] = op->herm == 1 ? rng.uniform() : 0.0;
  int N = s.norb;
  double f1 = 0.0;
  for (int i = 0; i < N; ++i)
    for (int k = 0; k < s.ob_count[i]; ++k) {
      int j = s.ob_list[s.ob_start[i] + k];
      if (j < i) continue;
      double v = rng.uniform();
      if (i == j) v = (op->herm == 1) ? v : 0.0;
      a[32 + (size_t)j * N + i] = v;
      a[32 + (size_t)i * N + j] = (i == j) ? v : sg * v;
      f1 += (i == j ? 1.0 : 2.0) * v * v;
    }
  if (f1 > 0)
    for (int t = 0; t < N * N; ++t) a[32 + t] /= std::sqrt(f1);
  for (int c = 0; c < s.nch; ++c) {
    int n = s.ch[c].n();
    double* b = a.data() + s.ch[c].off;
    double f = 0.0;
    for (int j = 0; j < n; ++j)
      for (int i = 0; i <= j; ++i) {
        double v = rng.uniform();
        if (i == j && op->herm != 1) v = 0.0;
        b[(size_t)j * n + i] = v;
        b[(size_t)i * n + j] = (i == j) ? v : sg * v;
        f += (i == j ? 1.0 : 2.0) * v * v;
      }
    if (f > 0) {
      double r = 1.0 / std::sqrt(f);
      for (size_t t = 0; t < (size_t)n * n; ++t) b[t] *= r;
    }
  }
  CUDA_TRY(cudaMemcpyAsync(op->d, a.data(), s.arena * sizeof(double), cudaMemcpyHostToDevice, S_(stream)));
  CUDA_TRY(cudaStreamSynchronize(S_(stream)));
  return IMSRG_OK;
}

#define TERM_PROLOGUE                        \
  int rc = check_ops(X, Y, Z);               \
  if (rc) return rc;                         \
  cudaStream_t st = S_(stream);

int imsrg_comm110ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  TERM_PROLOGUE
  return do_111_110(X, Y, Z, false, true, st);
}

int imsrg_comm220ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  TERM_PROLOGUE
  return do_220(X, Y, Z, st);
}

int imsrg_comm111ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  TERM_PROLOGUE
  return do_111_110(X, Y, Z, true, false, st);
}

int imsrg_comm121ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  TERM_PROLOGUE
  return do_121(X, Y, Z, st);
}

int imsrg_comm122ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  TERM_PROLOGUE
  return do_122(X, Y, Z, st);
}

int imsrg_comm221ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream)
{
  TERM_PROLOGUE
  return do_221_1b(X, Y, Z, st);
}

int imsrg_comm222_pp_hhss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  TERM_PROLOGUE
  rc = do_ladder(X, Y, Z, precision, st);
  if (rc == IMSRG_OK && precision == IMSRG_PREC_SPLIT) rc = end_status(X->sp, st);
  return rc;
}

int imsrg_comm222_pp_hh_221ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  TERM_PROLOGUE
  if ((rc = do_ladder(X, Y, Z, precision, st))) return rc;
  if ((rc = do_221_1b(X, Y, Z, st))) return rc;
  if (precision == IMSRG_PREC_SPLIT) rc = end_status(X->sp, st);
  return rc;
}

int imsrg_comm222_phss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  TERM_PROLOGUE
  rc = do_ph(X, Y, Z, precision, st);
  if (rc == IMSRG_OK && precision == IMSRG_PREC_SPLIT) rc = end_status(X->sp, st);
  return rc;
}

int imsrg_commutator_scalar_scalar(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream)
{
  int rc = commutator_impl(X, Y, Z, precision, S_(stream));
  if (rc == IMSRG_OK && precision == IMSRG_PREC_SPLIT) rc = end_status(X->sp, S_(stream));
  return rc;
}

int imsrg_space_zbar_layout(const imsrg_space* sp, int ch_cc, int* rows, int* cols, long long* offset,
                            long long* total)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "bad arguments");
  const Space& s = *sp->s;
  if (total) *total = std::max<int64_t>(1, s.zb_total);
  if (ch_cc < 0) return IMSRG_OK;
  if (ch_cc >= s.nch) return fail(IMSRG_ERR_ARG, "channel index out of range");
  if (rows) *rows = s.cc[ch_cc].n();
  if (cols) *cols = 2 * s.cc[ch_cc].n();
  if (offset) *offset = s.zb_off[ch_cc];
  return IMSRG_OK;
}

int imsrg_add_inverse_pandya(const double* zbar, imsrg_op* Z, int precision, void* stream)
{
  if (!zbar || !Z) return fail(IMSRG_ERR_ARG, "bad arguments");
  if (Z->tl) return fail(IMSRG_ERR_UNSUPPORTED, "Z must be a scalar operator");
  if (Z->herm != 1 && Z->herm != -1) return fail(IMSRG_ERR_UNSUPPORTED, "Z must be hermitian or anti-hermitian");
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_SPLIT) return fail(IMSRG_ERR_ARG, "bad precision");
  cudaStream_t st = S_(stream);
  ProfScope ps("InversePandyaTransformation", st);
  return inverse_pandya(Z->sp, zbar, Z->d, Z->herm, precision, st);
}

int imsrg_space_set_tuning(imsrg_space* sp, const char* name, int value)
{
  if (!sp || !name) return fail(IMSRG_ERR_ARG, "bad arguments");
  int t = tune_index(name);
  if (t < 0) return fail(IMSRG_ERR_ARG, std::string("unknown tuning parameter ") + name);
  std::lock_guard<std::mutex> g(sp->mu);
  int rc = tune_apply(sp, t, value);
  if (rc == IMSRG_OK) sp->tuning_source = "set";
  return rc;
}

int imsrg_space_get_tuning(const imsrg_space* sp, const char* name, int* value)
{
  if (!sp || !name || !value) return fail(IMSRG_ERR_ARG, "bad arguments");
  int t = tune_index(name);
  if (t < 0) return fail(IMSRG_ERR_ARG, std::string("unknown tuning parameter ") + name);
  int v = *tune_slot(const_cast<imsrg_space*>(sp), t);
  if (t == 0 && v == 0) v = 64;
  if (t == 3 && v == 0) v = 32;
  *value = v;
  return IMSRG_OK;
}

int imsrg_space_describe_tuning(const imsrg_space* sp, char* buf, int buflen)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "null space");
  std::string all = "source=" + sp->tuning_source;
  for (int t = 0; t < kNTune; ++t) {
    int v = 0;
    imsrg_space_get_tuning(sp, kTuneNames[t], &v);
    all += std::string(" ") + kTuneNames[t] + "=" + std::to_string(v);
  }
  if (!buf || buflen <= 0) return (int)all.size() + 1;
  int n = std::min<int>((int)all.size(), buflen - 1);
  all.copy(buf, n);
  buf[n] = 0;
  return IMSRG_OK;
}

int imsrg_space_defer_status(imsrg_space* sp, int defer)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "null space");
  sp->defer_status = defer != 0;
  return IMSRG_OK;
}

int imsrg_space_check_status(imsrg_space* sp, void* stream)
{
  if (!sp) return fail(IMSRG_ERR_ARG, "null space");
  if (!sp->dev_ready) return IMSRG_OK;  // nothing has run on the device
  return check_status(sp, S_(stream));
}

int imsrg_set_term(const char* name, int on)
{
  if (!name) return fail(IMSRG_ERR_ARG, "null name");
  std::lock_guard<std::mutex> g(g_mu);
  for (int t = 0; t < NTERMS; ++t)
    if (std::strcmp(name, kTermNames[t]) == 0) {
      g_term_on[t] = on != 0;
      return IMSRG_OK;
    }
  return fail(IMSRG_ERR_ARG, std::string("unknown term ") + name);
}

int imsrg_get_term(const char* name, int* on)
{
  if (!name || !on) return fail(IMSRG_ERR_ARG, "bad arguments");
  std::lock_guard<std::mutex> g(g_mu);
  for (int t = 0; t < NTERMS; ++t)
    if (std::strcmp(name, kTermNames[t]) == 0) {
      *on = g_term_on[t] ? 1 : 0;
      return IMSRG_OK;
    }
  return fail(IMSRG_ERR_ARG, std::string("unknown term ") + name);
}

int imsrg_set_default_precision(int precision)
{
  if (precision != IMSRG_PREC_FP64 && precision != IMSRG_PREC_SPLIT) return fail(IMSRG_ERR_ARG, "bad precision");
  std::lock_guard<std::mutex> g(g_mu);
  g_default_precision = precision;
  return IMSRG_OK;
}

int imsrg_get_default_precision(int* precision)
{
  if (!precision) return fail(IMSRG_ERR_ARG, "null pointer");
  std::lock_guard<std::mutex> g(g_mu);
  *precision = g_default_precision;
  return IMSRG_OK;
}

int imsrg_bch_transform(const imsrg_op* OpIn, const imsrg_op* Omega, imsrg_op* OpOut, double threshold,
                        int precision, int* n_nested, void* stream)
{
  if (!OpIn || !Omega || !OpOut) return fail(IMSRG_ERR_ARG, "null operator");
  if (OpIn->sp != Omega->sp || OpIn->sp != OpOut->sp) return fail(IMSRG_ERR_ARG, "different model spaces");
  if (Omega->tl) return fail(IMSRG_ERR_UNSUPPORTED, "Omega must be a scalar operator");
  if (OpOut->tl != OpIn->tl) return fail(IMSRG_ERR_ARG, "OpIn and OpOut must have the same rank");
  if (OpOut == Omega) return fail(IMSRG_ERR_ARG, "OpOut must not alias Omega");
  if ((Omega->herm != 1 && Omega->herm != -1) || (OpIn->herm != 1 && OpIn->herm != -1))
    return fail(IMSRG_ERR_UNSUPPORTED, "operators must be hermitian or anti-hermitian");
  cudaStream_t st = S_(stream);
  if (OpIn->tl) return tensor_bch_transform(OpIn, Omega, OpOut, threshold, precision, n_nested, st);
  imsrg_space* sp = OpIn->sp;
  if (n_nested) *n_nested = 0;
  int rc;
  double nx = 0, ny = 0;
  if ((rc = norm_impl(OpIn, &nx, st))) return rc;
  if ((rc = norm_impl(Omega, &ny, st))) return rc;
  if ((rc = imsrg_op_copy(OpOut, OpIn, stream))) return rc;
  if (!(nx > threshold)) return IMSRG_OK;
  try {
    if (!sp->d_nested) sp->d_nested = sp->track(dmalloc<double>(sp->s->arena));
    if (!sp->d_next) sp->d_next = sp->track(dmalloc<double>(sp->s->arena));
  } catch (std::exception&) {
    return fail(IMSRG_ERR_NOMEM, "BCH work operators");
  }
  imsrg_op nested, next;
  nested.sp = next.sp = sp;
  nested.d = sp->d_nested;
  next.d = sp->d_next;
  CUDA_TRY(cudaMemcpyAsync(nested.d, OpOut->d, sp->s->arena * sizeof(double), cudaMemcpyDeviceToDevice, st));
  nested.herm = OpOut->herm;
  double epsilon = nx * std::exp(-2 * ny) * threshold / (2 * ny);
  double fden = 1.0;
  for (int i = 1; i <= 40; ++i) {
    if ((rc = commutator_impl(Omega, &nested, &next, precision, st))) return rc;
    std::swap(nested.d, next.d);
    std::swap(nested.herm, next.herm);
    fden /= i;
    // OpOut += fden nested and the norm of nested in one pass, then one
    // host sync for the norm and (split form) the kernels' status word
    CUDA_TRY(launch_axpy_norm(*sp->s, OpOut->d, nested.d, fden, sp->d_norm_off, sp->d_norm_len, sp->d_norm_w,
                              sp->n_norm, sp->d_norm_partial, st));
    if (n_nested) *n_nested = i;
    epsilon *= i + 1;
    CUDA_TRY(cudaMemcpyAsync(sp->h_norm_partial.data(), sp->d_norm_partial, (sp->n_norm + 1) * sizeof(double),
                             cudaMemcpyDeviceToHost, st));
    int hstat = 0;
    if (precision == IMSRG_PREC_SPLIT)
      CUDA_TRY(cudaMemcpyAsync(&hstat, sp->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (hstat != 0) {
      cudaMemsetAsync(sp->d_status, 0, sizeof(int), st);
      return fail(IMSRG_ERR_KERNEL, "a kernel reported error status " + std::to_string(hstat));
    }
    double n2 = 0.0;
    for (int c = 0; c < sp->n_norm; ++c) n2 += sp->h_norm_partial[c];
    const double nn = std::sqrt(sp->h_norm_partial[sp->n_norm] + n2);
    if (nn < epsilon) break;
  }
  return IMSRG_OK;
}

}  // extern "C"

// entry points of this file the flow layer (capi_flow.cu) builds on
namespace imsrg {
int commutator_dev(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int prec, cudaStream_t st)
{
  return commutator_impl(X, Y, Z, prec, st);
}
int norm_dev(const imsrg_op* op, double* out, cudaStream_t st) { return norm_impl(op, out, st); }
int status_dev(imsrg_space* sp, cudaStream_t st) { return check_status(sp, st); }
int end_status(imsrg_space* sp, cudaStream_t st) { return sp->defer_status ? IMSRG_OK : check_status(sp, st); }
}  // namespace imsrg

// ------------------------------------------------------------- batch phases
// CommutatorScalarScalar in the split form for a group of pairs of the same
// structure, every kernel launched once for all of them (see capi_batch.cu):
// pre (Z zeroed, operand preparation, the zero- and one-body terms), the
// ladder product, mid (comm221ss, comm122ss), the Zbar product, post (inverse
// Pandya transform).  Every term must be on.
namespace imsrg {

bool batch_phases_usable()
{
  std::lock_guard<std::mutex> g(g_mu);
  for (int t = 0; t < NSCALAR_TERMS; ++t)
    if (!g_term_on[t]) return false;
  return true;
}

void tensor_terms_on(bool on[5])
{
  std::lock_guard<std::mutex> g(g_mu);
  on[0] = g_term_on[TS111];
  on[1] = g_term_on[TS121];
  on[2] = g_term_on[TS122];
  on[3] = g_term_on[TS222PPHH] && g_term_on[TS221];
  on[4] = g_term_on[TS222PH];
}

// Products of several pairs whose spaces have the same structure (equal
// orbit lists, hence equal channel tables and product job lists) and whose
// operators have the same hermiticities, as one split-form launch per
// product family.  The jobs of pair p address its own operands: every job
// offset is moved by the distance, in doubles, from pair 0's operand to pair
// p's (all operands are 8-byte aligned device allocations), so the kernels
// run unchanged on pair 0's base pointers, and the digit splitting (chosen
// from K) is the one each pair's own plan makes.
struct GroupedProducts {
  std::vector<const imsrg_op*> X, Y;
  std::vector<imsrg_op*> Z;
  int prec = IMSRG_PREC_SPLIT;
  SplitPlan* ladder = nullptr;  // split form
  SplitPlan* zbar = nullptr;
  // FP64 form: every pair's jobs and tile pairs in one list per product
  GemmJobDev *d_lj = nullptr, *d_zj = nullptr;
  int *d_lp = nullptr, *d_zp = nullptr;
  int n_lp = 0, n_zp = 0;
  // byte offsets of every pair's operands and scratch from pair 0's, for
  // the grouped launches of the other kernels (kZRoles per pair)
  long long* d_zoff = nullptr;
  ~GroupedProducts()
  {
    if (ladder) split_plan_destroy(ladder);
    if (zbar) split_plan_destroy(zbar);
    if (d_zoff) cudaFree(d_zoff);
    for (void* p : {(void*)d_lj, (void*)d_zj, (void*)d_lp, (void*)d_zp})
      if (p) cudaFree(p);
  }
};

static long long bdist(const void* a, const void* b) { return (long long)(intptr_t)a - (long long)(intptr_t)b; }

static long long dist(const void* a, const void* b)
{
  return ((long long)(intptr_t)a - (long long)(intptr_t)b) / (long long)sizeof(double);
}

GroupedProducts* grouped_products_create(const std::vector<const imsrg_op*>& X, const std::vector<const imsrg_op*>& Y,
                                         const std::vector<imsrg_op*>& Z, int prec, std::string* why)
{
  if (X.empty()) return nullptr;
  imsrg_space* s0 = X[0]->sp;
  for (size_t p = 0; p < X.size(); ++p) {
    imsrg_space* sp = X[p]->sp;
    if (sp->s->norb != s0->s->norb || sp->s->arena != s0->s->arena || sp->s->emax != s0->s->emax ||
        sp->ladder_jobs.size() != s0->ladder_jobs.size() || sp->zbar_jobs.size() != s0->zbar_jobs.size() ||
        X[p]->herm != X[0]->herm || Y[p]->herm != Y[0]->herm || !sp->d_zb || !sp->d_xb) {
      if (why) *why = "pairs differ in structure or hermiticity";
      return nullptr;
    }
  }
  std::vector<GemmJobDev> lj, zj;
  for (size_t p = 0; p < X.size(); ++p) {
    imsrg_space* sp = X[p]->sp;
    const long long dX = dist(X[p]->d, X[0]->d), dY = dist(Y[p]->d, Y[0]->d), dZ = dist(Z[p]->d, Z[0]->d);
    for (GemmJobDev j : sp->ladder_jobs) {
      j.a_off += dX;
      j.b_off += dY;  // B0 = B1 = Y
      j.out_off += dZ;
      lj.push_back(j);
    }
    const long long dA = dist(sp->d_xb, s0->d_xb), dB0 = dist(sp->d_yt, s0->d_yt), dB1 = dist(sp->d_yf, s0->d_yf),
                    dO = dist(sp->d_zb, s0->d_zb);
    for (GemmJobDev j : sp->zbar_jobs) {
      j.a_off += dA;
      j.b_off += j.bsel ? dB1 : dB0;
      j.out_off += dO;
      zj.push_back(j);
    }
  }
  if (prec == IMSRG_PREC_FP64 && s0->inv_fp64 == 0) {
    if (why) *why = "the FP64 form's grouped inverse Pandya needs the descriptor kernel (inverse.fp64 = 1)";
    return nullptr;
  }
  GroupedProducts* g = new GroupedProducts();
  g->X = X;
  g->Y = Y;
  g->Z = Z;
  g->prec = prec;
  std::vector<long long> zo;
  for (size_t p = 0; p < X.size(); ++p) {
    imsrg_space* sp = X[p]->sp;
    long long r[kZRoles];
    r[ZR_X] = bdist(X[p]->d, X[0]->d);
    r[ZR_Y] = bdist(Y[p]->d, Y[0]->d);
    r[ZR_Z] = bdist(Z[p]->d, Z[0]->d);
    r[ZR_XF] = bdist(sp->d_xf, s0->d_xf);
    r[ZR_YF] = bdist(sp->d_yff, s0->d_yff);
    r[ZR_W2] = bdist(sp->d_w2, s0->d_w2);
    r[ZR_XB] = bdist(sp->d_xb, s0->d_xb);
    r[ZR_YT] = bdist(sp->d_yt, s0->d_yt);
    r[ZR_YFL] = bdist(sp->d_yf, s0->d_yf);
    r[ZR_ZB] = bdist(sp->d_zb, s0->d_zb);
    zo.insert(zo.end(), r, r + kZRoles);
  }
  try {
    if (prec == IMSRG_PREC_SPLIT) {
      g->ladder = split_plan_create(*s0->s, lj, 0, s0->opt_ladder);
      g->zbar = split_plan_create(*s0->s, zj, 1, s0->opt_zbar);
    } else {
      // the FP64 products' tile pairs over every pair's jobs (offsets from pair 0's arrays)
      std::vector<int> lp = tile_pairs(lj, symgemm_fp64_tile()), zp = tile_pairs(zj, symgemm_fp64_tile());
      g->d_lj = dcopy(lj);
      g->d_zj = dcopy(zj);
      g->d_lp = dcopy(lp);
      g->d_zp = dcopy(zp);
      g->n_lp = (int)lp.size() / 3;
      g->n_zp = (int)zp.size() / 3;
    }
    g->d_zoff = dcopy(zo);
  } catch (std::exception& e) {
    if (why) *why = std::string("grouped product plans: ") + e.what();
    delete g;
    return nullptr;
  }
  return g;
}

// the per-pair phases of a group as one launch per kernel (the grid's z is the pair)
int group_pre(GroupedProducts* g, cudaStream_t st)
{
  const int nz = (int)g->X.size();
  for (int p = 0; p < nz; ++p) {
    imsrg_space* sp = g->X[p]->sp;
    g->Z[p]->herm = z_herm(g->X[p]->herm, g->Y[p]->herm);
    CUDA_TRY(cudaMemsetAsync(g->Z[p]->d, 0, sp->s->arena * sizeof(double), st));
    for (auto& zr : sp->zbar_zero) CUDA_TRY(cudaMemsetAsync(sp->d_zb + zr.first, 0, zr.second * sizeof(double), st));
  }
  const imsrg_op *X = g->X[0], *Y = g->Y[0];
  imsrg_op* Z = g->Z[0];
  imsrg_space* sp = X->sp;
  const Space& s = *sp->s;
  const long long* zo = g->d_zoff;
  if (g->prec == IMSRG_PREC_SPLIT) {
    CUDA_TRY(launch_to_ff(s, X->d, sp->d_xf, st, zo, nz, ZR_X, ZR_XF));
    CUDA_TRY(launch_to_ff(s, Y->d, sp->d_yff, st, zo, nz, ZR_Y, ZR_YF));
  }
  CUDA_TRY(launch_pandya_fwd(s, X->d, Y->d, Y->herm, sp->d_xb, sp->d_yt, sp->d_yf, g->prec == IMSRG_PREC_SPLIT, st,
                             zo, nz));
  CUDA_TRY(launch_comm111_110(s, X->d, Y->d, Z->d, true, X->herm != Y->herm, st, zo, nz));
  if (X->herm != Y->herm) CUDA_TRY(launch_comm220(s, X->d, Y->d, Z->d, X->herm, st, zo, nz));
  CUDA_TRY(launch_comm121(s, sp->d_holes, X->d, Y->d, Z->d, Z->herm, st, zo, nz));
  return IMSRG_OK;
}

int group_mid(GroupedProducts* g, cudaStream_t st)
{
  const int nz = (int)g->X.size();
  const imsrg_op *X = g->X[0], *Y = g->Y[0];
  imsrg_op* Z = g->Z[0];
  imsrg_space* sp = X->sp;
  const Space& s = *sp->s;
  const long long* zo = g->d_zoff;
  CUDA_TRY(launch_comm221_1b(s, X->d, Y->d, Z->d, X->herm, Z->herm, Z->d, st, zo, nz));
  if (g->prec == IMSRG_PREC_FP64)
    CUDA_TRY(launch_comm122(s, X->d, Y->d, Z->d, sp->d_w2, Z->herm, sp->d_sym122, sp->n_sym122, st, zo, nz));
  else if (sp->comm122_fused)
    CUDA_TRY(launch_comm122_fused_df(s, X->d, Y->d, Z->d, sp->d_xf, sp->d_yff, Z->herm, sp->d_sym122u, sp->n_sym122u,
                                     st, zo, nz));
  else
    CUDA_TRY(launch_comm122_df(s, X->d, Y->d, Z->d, sp->d_xf, sp->d_yff, (float2*)sp->d_w2, Z->herm, sp->d_sym122,
                               sp->n_sym122, st, zo, nz));
  return IMSRG_OK;
}

int group_post(GroupedProducts* g, cudaStream_t st)
{
  const int nz = (int)g->X.size();
  imsrg_op* Z = g->Z[0];
  imsrg_space* sp = g->X[0]->sp;
  const Space& s = *sp->s;
  if (g->prec == IMSRG_PREC_FP64 || sp->inv_split != 0 || sp->n_invq > 0) {
    int rc = inverse_pandya(sp, sp->d_zb, Z->d, Z->herm, g->prec, st, g->d_zoff, nz);
    if (rc) return rc;
  } else {
    for (int p = 0; p < nz; ++p) {
      imsrg_space* q = g->X[p]->sp;
      CUDA_TRY(launch_pandya_inv(*q->s, q->d_zb, g->Z[p]->d, g->Z[p]->herm, q->d_pinv, q->n_pinv, st));
    }
  }
  return IMSRG_OK;
}

void grouped_products_destroy(GroupedProducts* g) { delete g; }

int grouped_ladder(GroupedProducts* g, cudaStream_t st)
{
  imsrg_space* s0 = g->X[0]->sp;
  const Space& s = *s0->s;
  if (g->prec == IMSRG_PREC_FP64) {
    CUDA_TRY(launch_symgemm_fp64(g->d_lj, g->d_lp, g->n_lp, g->X[0]->d, g->Y[0]->d, g->Y[0]->d, g->Z[0]->d,
                                 s.work.kidx, s.work.kweight, s.work.phase_tab, g->Z[0]->herm,
                                 (double)g->Y[0]->herm, st));
    return IMSRG_OK;
  }
  split_plan_set_accumulate(g->ladder, 0);  // Z was zeroed in the pre phase
  CUDA_TRY(launch_symgemm_split(g->ladder, g->X[0]->d, g->Y[0]->d, g->Y[0]->d, g->Z[0]->d, s.work.kidx,
                                s.work.kweight, s.work.phase_tab, s0->d_status, g->Z[0]->herm,
                                (double)g->Y[0]->herm, st));
  return IMSRG_OK;
}

int grouped_zbar(GroupedProducts* g, cudaStream_t st)
{
  imsrg_space* s0 = g->X[0]->sp;
  const Space& s = *s0->s;
  if (g->prec == IMSRG_PREC_FP64) {
    CUDA_TRY(launch_symgemm_fp64(g->d_zj, g->d_zp, g->n_zp, s0->d_xb, s0->d_yt, s0->d_yf, s0->d_zb, s.work.kidx,
                                 s.work.kweight, s.work.phase_tab, g->Z[0]->herm, 1.0, st));
    return IMSRG_OK;
  }
  split_plan_set_mirror(g->zbar, s0->inv_split == 0 ? 1 : 0);  // as group_post reads Zbar
  CUDA_TRY(launch_symgemm_split(g->zbar, s0->d_xb, s0->d_yt, s0->d_yf, s0->d_zb, s.work.kidx, s.work.kweight,
                                s.work.phase_tab, s0->d_status, g->Z[0]->herm, 1.0, st));
  return IMSRG_OK;
}

}  // namespace imsrg
