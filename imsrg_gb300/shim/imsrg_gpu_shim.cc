// Drop-in shim: IMSRG++'s Commutator::comm*ss, Commutator::CommutatorScalarScalar
// and BCH::Standard_BCH_Transform with their reference signatures
// (src/Commutator.hh:57-87, src/BCH.hh:22-25), evaluated by libimsrg_gb300.
//
// Compiled against the reference's own headers and linked in place of the
// same functions of the reference's Commutator.o / BCH.o, the rest of IMSRG++
// (the other commutators, IMSRGSolver, UnitTest) runs unchanged on top of the
// GPU path.  oracle/ref_build.mk (target shim) does that link.
//
// Each call packs the reference Operators into arenas (one memcpy per
// TwoBodyME block: the arena blocks are arma::mat's memory order), uploads
// them, runs the C ABI entry point and copies Z back.  Z keeps the reference
// semantics: the terms accumulate into the caller's Z, CommutatorScalarScalar
// returns a new Operator whose hermiticity is set from X and Y.  The
// precision of the dense products is imsrg_set_default_precision's
// (process-wide, FP64 unless changed).  Errors of the GPU path throw
// std::runtime_error (the reference itself exits on unsupported symmetries).
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "BCH.hh"
#include "Commutator.hh"
#include "ModelSpace.hh"
#include "Operator.hh"
#include "imsrg_gb300.h"

namespace {

struct GpuSpace {  // one per reference ModelSpace
  imsrg_space* s = nullptr;
  long long arena = 0;
  std::vector<long long> off;  // scalar arena offset of each two-body channel
};
std::mutex g_mu;
std::map<const ModelSpace*, GpuSpace> g_spaces;

void ok(int rc)
{
  if (rc != IMSRG_OK) throw std::runtime_error(std::string("imsrg_gb300: ") + imsrg_last_error());
}

// the GPU model space of a reference ModelSpace: the same orbit list, so the
// same channels and ket order (the arena layout then equals the reference's
// TwoBodyME blocks)
GpuSpace& space_of(ModelSpace& ms)
{
  std::lock_guard<std::mutex> g(g_mu);
  auto it = g_spaces.find(&ms);
  if (it != g_spaces.end()) return it->second;
  GpuSpace gs;
  const int norb = ms.GetNumberOrbits();
  std::vector<int> n(norb), l(norb), j2(norb), tz2(norb);
  std::vector<double> occ(norb);
  for (int i = 0; i < norb; ++i) {
    Orbit& o = ms.GetOrbit(i);
    n[i] = o.n;
    l[i] = o.l;
    j2[i] = o.j2;
    tz2[i] = o.tz2;
    occ[i] = o.occ;
  }
  ok(imsrg_space_create(ms.GetEmax(), norb, n.data(), l.data(), j2.data(), tz2.data(), occ.data(), &gs.s));
  int nch = 0;
  ok(imsrg_space_sizes(gs.s, nullptr, &nch, &gs.arena));
  if (nch != ms.GetNumberTwoBodyChannels()) throw std::runtime_error("imsrg_gb300: channel count differs");
  gs.off.resize(nch);
  for (int ch = 0; ch < nch; ++ch) ok(imsrg_space_channel(gs.s, ch, nullptr, nullptr, nullptr, nullptr, &gs.off[ch]));
  return g_spaces[&ms] = gs;
}

int herm_of(const Operator& op)
{
  if (op.IsHermitian()) return 1;
  if (op.IsAntiHermitian()) return -1;
  throw std::runtime_error("imsrg_gb300: the GPU path takes hermitian or anti-hermitian operators");
}

bool is_scalar(const Operator& op) { return op.GetJRank() == 0 && op.GetTRank() == 0 && op.GetParity() == 0; }

// a device operator of op's rank, with op's elements
struct DevOp {
  imsrg_op* d = nullptr;
  long long len = 0;
  std::map<std::array<size_t, 2>, long long> off;  // block offsets
  DevOp(GpuSpace& gs, const Operator& op, bool upload)
  {
    if (op.GetParticleRank() > 2) throw std::runtime_error("imsrg_gb300: particle rank > 2 is not on the GPU path");
    if (is_scalar(op)) {
      ok(imsrg_op_create(gs.s, herm_of(op), &d));
      len = gs.arena;
      for (size_t ch = 0; ch < gs.off.size(); ++ch) off[{ch, ch}] = gs.off[ch];
    } else {
      ok(imsrg_op_create_tensor(gs.s, op.GetJRank(), op.GetTRank(), op.GetParity(), herm_of(op), &d));
      int nb = 0;
      ok(imsrg_space_tensor_layout(gs.s, op.GetJRank(), op.GetTRank(), op.GetParity(), -1, nullptr, nullptr,
                                   nullptr, &nb, &len));
      for (int b = 0; b < nb; ++b) {
        int cb = 0, ck = 0;
        long long o = 0;
        ok(imsrg_space_tensor_layout(gs.s, op.GetJRank(), op.GetTRank(), op.GetParity(), b, &cb, &ck, &o, nullptr,
                                     nullptr));
        off[{(size_t)cb, (size_t)ck}] = o;
      }
    }
    if (upload) {
      std::vector<double> a((size_t)len, 0.0);
      const size_t N = op.OneBody.n_rows;
      a[0] = op.ZeroBody;
      std::memcpy(&a[32], op.OneBody.memptr(), N * N * sizeof(double));
      for (auto& it : op.TwoBody.MatEl) {
        auto o = off.find(it.first);
        if (o == off.end()) throw std::runtime_error("imsrg_gb300: two-body block outside the arena layout");
        std::memcpy(&a[(size_t)o->second], it.second.memptr(), it.second.n_elem * sizeof(double));
      }
      ok(imsrg_op_upload(d, a.data(), nullptr));
    }
  }
  void download(Operator& op)
  {
    std::vector<double> a((size_t)len);
    ok(imsrg_op_download(d, a.data(), nullptr));
    const size_t N = op.OneBody.n_rows;
    op.ZeroBody = a[0];
    std::memcpy(op.OneBody.memptr(), &a[32], N * N * sizeof(double));
    for (auto& it : op.TwoBody.MatEl) {
      auto o = off.find(it.first);
      if (o == off.end()) throw std::runtime_error("imsrg_gb300: two-body block outside the arena layout");
      std::memcpy(it.second.memptr(), &a[(size_t)o->second], it.second.n_elem * sizeof(double));
    }
    int h = 1;
    ok(imsrg_op_hermiticity(d, &h));
    if (h == 1)
      op.SetHermitian();
    else
      op.SetAntiHermitian();
  }
  ~DevOp() { imsrg_op_destroy(d); }
  DevOp(const DevOp&) = delete;
  DevOp& operator=(const DevOp&) = delete;
};

int precision()
{
  int p = IMSRG_PREC_FP64;
  imsrg_get_default_precision(&p);
  return p;
}

// a term: X, Y, Z uploaded, fn(x, y, z) accumulates into z, Z copied back
template <class F>
void term(const Operator& X, const Operator& Y, Operator& Z, F fn)
{
  if (!is_scalar(X) || !is_scalar(Y) || !is_scalar(Z))
    throw std::runtime_error("imsrg_gb300: the comm*ss terms take scalar operators");
  GpuSpace& gs = space_of(*X.modelspace);
  DevOp x(gs, X, true), y(gs, Y, true), z(gs, Z, true);
  ok(fn(x.d, y.d, z.d));
  z.download(Z);
}

}  // namespace

namespace Commutator {

void comm110ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm110ss(x, y, z, nullptr); });
}
void comm220ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm220ss(x, y, z, nullptr); });
}
void comm111ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm111ss(x, y, z, nullptr); });
}
void comm121ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm121ss(x, y, z, nullptr); });
}
void comm122ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm122ss(x, y, z, nullptr); });
}
void comm221ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm221ss(x, y, z, nullptr); });
}
void comm222_pp_hhss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z,
       [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm222_pp_hhss(x, y, z, precision(), nullptr); });
}
void comm222_pp_hh_221ss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z, [](imsrg_op* x, imsrg_op* y, imsrg_op* z) {
    return imsrg_comm222_pp_hh_221ss(x, y, z, precision(), nullptr);
  });
}
void comm222_phss(const Operator& X, const Operator& Y, Operator& Z)
{
  term(X, Y, Z,
       [](imsrg_op* x, imsrg_op* y, imsrg_op* z) { return imsrg_comm222_phss(x, y, z, precision(), nullptr); });
}

// src/Commutator.cc:280-428: Z = [X, Y] in IMSRG(2), hermiticity from X and
// Y, the terms switched on in comm_term_on (forwarded to imsrg_set_term)
Operator CommutatorScalarScalar(const Operator& X, const Operator& Y)
{
  static const char* names[] = {"comm110ss",  "comm220ss",  "comm111ss",       "comm121ss",
                                "comm122ss",  "comm221ss",  "comm222_pp_hhss", "comm222_phss"};
  for (const char* n : names) {
    auto it = comm_term_on.find(n);
    ok(imsrg_set_term(n, it == comm_term_on.end() || it->second ? 1 : 0));
  }
  Operator Z(*X.modelspace, 0, 0, 0, 2);
  if (X.IsHermitian() == Y.IsHermitian())
    Z.SetAntiHermitian();
  else
    Z.SetHermitian();
  GpuSpace& gs = space_of(*X.modelspace);
  DevOp x(gs, X, true), y(gs, Y, true), z(gs, Z, false);
  ok(imsrg_commutator_scalar_scalar(x.d, y.d, z.d, precision(), nullptr));
  z.download(Z);
  return Z;
}

}  // namespace Commutator

namespace BCH {

// src/BCH.cc:87-201: OpOut = e^Omega Op e^-Omega by nested commutators that
// stay in device memory, with the reference's stopping rule and threshold
// (bch_transform_threshold)
Operator Standard_BCH_Transform(const Operator& Op, const Operator& Omega)
{
  if (!is_scalar(Omega)) throw std::runtime_error("imsrg_gb300: Omega must be a scalar operator");
  GpuSpace& gs = space_of(*Op.modelspace);
  DevOp in(gs, Op, true), om(gs, Omega, true), out(gs, Op, false);
  int nested = 0;
  ok(imsrg_bch_transform(in.d, om.d, out.d, bch_transform_threshold, precision(), &nested, nullptr));
  Operator OpOut = Op;
  out.download(OpOut);
  return OpOut;
}

}  // namespace BCH

// The layout check the shim's link test runs without a GPU: for every channel
// of ModelSpace(emax, ref, ref), the GPU space's kets must be the reference's
// TwoBodyChannel kets in the same order.  Returns the number of mismatches.
extern "C" int imsrg_gpu_shim_layout_check(ModelSpace* ms)
{
  GpuSpace& gs = space_of(*ms);
  int bad = 0;
  const int nch = ms->GetNumberTwoBodyChannels();
  for (int ch = 0; ch < nch; ++ch) {
    TwoBodyChannel& tbc = ms->GetTwoBodyChannel(ch);
    int J = 0, par = 0, Tz = 0, nk = 0;
    long long off = 0;
    ok(imsrg_space_channel(gs.s, ch, &J, &par, &Tz, &nk, &off));
    if (J != tbc.J || par != tbc.parity || Tz != tbc.Tz || nk != tbc.GetNumberKets()) {
      ++bad;
      continue;
    }
    std::vector<int> p(nk > 0 ? nk : 1), q(nk > 0 ? nk : 1);
    if (nk) ok(imsrg_space_channel_kets(gs.s, ch, p.data(), q.data()));
    for (int i = 0; i < nk; ++i)
      if (p[i] != tbc.GetKet(i).p || q[i] != tbc.GetKet(i).q) ++bad;
  }
  return bad;
}
