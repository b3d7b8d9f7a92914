// Model-space bookkeeping, restating the reference's rules:
//   orbit order + reference occupations  ModelSpace::Init, GetOrbitsAZ
//                                        (src/ModelSpace.cc:353-417, 610-645)
//   kets p <= q, Index2, pp/hh/ph        ModelSpace::SetupKets (src/ModelSpace.cc:1108-1200)
//   2b channel membership                TwoBodyChannel::CheckChannel_ket (src/TwoBodyChannel.cc:142-151)
//   cross-coupled channel membership     TwoBodyChannel_CC::CheckChannel_ket (src/TwoBodyChannel.cc:180-188)
//   channel index 6J + 2(Tz+1) + parity  ModelSpace::GetTwoBodyChannelIndex (src/ModelSpace.cc:1046-1053)
// plus the arena layout and the per-kernel work lists.
#include "space.hpp"
#include "tensor.hpp"

#include <algorithm>
#include <cstdint>
#include <cmath>
#include <cstdlib>
#include <map>
#include <stdexcept>

#include <cuda_runtime.h>

namespace imsrg {

static const double OCC_CUT = 1e-6;  // ModelSpace::OCC_CUT (src/ModelSpace.cc:14)

static int64_t round32(int64_t x) { return (x + 31) / 32 * 32; }

void reference_orbits(int emax, int A, int Z, std::vector<int>& n, std::vector<int>& l, std::vector<int>& j2,
                      std::vector<int>& tz2, std::vector<double>& occ)
{
  // occupations: fill proton and neutron shells in the order of GetOrbitsAZ
  std::map<std::vector<int>, double> filled;
  double zz = 0, nn = 0;
  bool done = false;
  for (int N = 0; N <= emax && !done; ++N) {
    for (int g = 2 * N + 1; g >= -2 * N; g -= 4) {
      int jj = std::abs(g);
      int ll = g < 0 ? (jj + 1) / 2 : (jj - 1) / 2;
      int nr = (N - ll) / 2;
      if (zz < Z) {
        double dz = std::min(Z - zz, jj + 1.0);
        filled[{nr, ll, jj, -1}] = dz / (jj + 1.0);
        zz += dz;
      }
      if (nn < A - Z) {
        double dn = std::min(A - Z - nn, jj + 1.0);
        filled[{nr, ll, jj, 1}] = dn / (jj + 1.0);
        nn += dn;
      }
      if (zz == Z && nn == A - Z) {
        done = true;
        break;
      }
    }
  }
  if (!done) throw std::runtime_error("model space too small for the reference nucleus");
  n.clear(); l.clear(); j2.clear(); tz2.clear(); occ.clear();
  for (int N = 0; N <= emax; ++N)
    for (int ll = N; ll >= 0; ll -= 2) {
      int nr = (N - ll) / 2;
      for (int jj = 2 * ll + 1; jj >= 2 * ll - 1 && jj > 0; jj -= 2)
        for (int tz : {-1, 1}) {
          n.push_back(nr);
          l.push_back(ll);
          j2.push_back(jj);
          tz2.push_back(tz);
          auto it = filled.find({nr, ll, jj, tz});
          occ.push_back(it == filled.end() ? 0.0 : it->second);
        }
    }
}

// Descriptors of the Pandya transform of X and Y
// (DoPandyaTransformation_SingleChannel_XandY, src/Commutator.cc:1392-1485, and
// the flipped Ybar of comm222_phss, src/Commutator.cc:1766-1788).  For every
// element (ik, t) of a cross-coupled channel's panels, t over its hh and ph
// bras and their swapped copies:
//   Xbar(ik, t) = normfactor (n_a - n_b) sum_J w_J X(e_J),
//   Ybar(t, ik) = normfactor             sum_J w_J Y(e_J),
// with w_J = -(2J+1) {j_a j_b J_cc; j_c j_d J} and the swap phases of
// GetTBME_J_norm folded into its sign, and e_J the arena index of the
// normalised J-coupled element (c b | a d).  Everything but X and Y is a
// property of the space, so it is listed once: the kernel is then one gather
// and FMA per term, in the same order as the J loop it replaces.
static void build_pandya_fwd(Space& s)
{
  constexpr double kSqrt2 = 1.4142135623730950488;
  // one task per (channel, bra column t): a run of n_cc consecutive outputs
  std::vector<std::pair<int, int>> tasks;
  for (int cc = 0; cc < s.nch; ++cc)
    if (s.cc[cc].n() > 0)
      for (int t = 0; t < 2 * s.cc_nph[cc]; ++t) tasks.push_back({cc, t});
  const int ntask = (int)tasks.size();
  std::vector<std::vector<PfOut>> outs(ntask);
  std::vector<std::vector<int>> es(ntask);
  std::vector<std::vector<double>> ws(ntask);
  bool too_big = false;
#pragma omp parallel for schedule(dynamic, 4)
  for (int task = 0; task < ntask; ++task) {
    const int cc = tasks[task].first, t = tasks[task].second;
    const Chan& K = s.cc[cc];
    const int ncc = K.n(), nph = s.cc_nph[cc];
    const int Jcc = cc / 6;
    const int* phi = s.phase_tab.data() + s.cc_phase_off[cc];
    const int ibra = t < nph ? t : t - nph;
    const int kb = s.cc_ph[s.cc_ph_off[cc] + ibra];
    const int a = t < nph ? K.p[kb] : K.q[kb], b = t < nph ? K.q[kb] : K.p[kb];
    const int tf = t < nph ? t + nph : t - nph;
    std::vector<PfOut>& out = outs[task];
    std::vector<int>& te = es[task];
    std::vector<double>& tw = ws[task];
    out.reserve(ncc);
    for (int ik = 0; ik < ncc; ++ik) {
      const int c = K.p[ik], d = K.q[ik];
      PfOut o{};
      const int64_t dest = s.xb_off[cc] + (int64_t)t * ncc + ik;
      if (dest > INT32_MAX) too_big = true;
      o.dest = (int)dest;
      o.dyf = (tf - t) * ncc;
      o.beg = (int)te.size();
      double nf = 1.0;
      unsigned nsq = 0;
      if (s.tz2[a] + s.tz2[d] == s.tz2[b] + s.tz2[c]) {
        if (a == d) nf *= kSqrt2, ++nsq;
        if (c == b) nf *= kSqrt2, ++nsq;
        const int ja = s.j2[a], jb = s.j2[b], jc = s.j2[c], jd = s.j2[d];
        int jmin = std::max(std::abs(ja - jd), std::abs(jc - jb)) / 2;
        const int jmax = std::min(ja + jd, jc + jb) / 2;
        int dJ = 1;
        if (a == d || c == b) {
          dJ = 2;
          jmin += jmin & 1;
        }
        const int lc = s.l[c], lb = s.l[b], la = s.l[a], ld = s.l[d];
        const bool ok = (((lc + lb + la + ld) & 1) == 0) && (s.tz2[c] + s.tz2[b] == s.tz2[a] + s.tz2[d]);
        if (ok) {
          const int k1 = ket_index(s.norb, std::min(c, b), std::max(c, b));
          const int k2 = ket_index(s.norb, std::min(a, d), std::max(a, d));
          const int par = (lc + lb) & 1, tz = (s.tz2[c] + s.tz2[b]) / 2;
          const int pcb = (c > b) ? ((jc + jb) / 2 + 1) : 0;
          const int pad = (a > d) ? ((ja + jd) / 2 + 1) : 0;
          for (int J = jmin; J <= jmax && J < s.NJ; J += dJ) {
            const int slot = sixj_slot(s.d1, s.sixj_base.data(), ja, jb, Jcc, jc, jd, J);
            const double w = slot < 0 ? 0.0 : s.sixj_wval[slot];
            if (w == 0.0) continue;
            const int bi = s.ketJ_loc[(size_t)J * s.nkets + k1], ki = s.ketJ_loc[(size_t)J * s.nkets + k2];
            if (bi < 0 || ki < 0) continue;
            const Chan& C = s.ch[chan_index(J, par, tz)];
            const int64_t e = C.off + (int64_t)ki * C.n() + bi;
            if (e > INT32_MAX) too_big = true;
            const bool neg = ((c > b) && ((pcb + J) & 1)) != ((a > d) && ((pad + J) & 1));
            te.push_back((int)e);
            tw.push_back(neg ? w : -w);  // -(2J+1) 6j with the swap phases
          }
        }
      }
      o.code = (unsigned)(te.size() - o.beg) | nsq << 16 | (phi[kb] * phi[ik] < 0 ? 1u : 0u) << 18;
      o.xs = nf * (s.occ[a] - s.occ[b]);
      out.push_back(o);
    }
  }
  if (too_big) throw std::runtime_error("Pandya transform descriptors: arena index beyond 2^31");
  size_t nout = 0, nterm = 0;
  for (int task = 0; task < ntask; ++task) {
    nout += outs[task].size();
    nterm += es[task].size();
  }
  if (nterm > (size_t)INT32_MAX) throw std::runtime_error("Pandya transform descriptors: more than 2^31 terms");
  s.pf_out.clear();
  s.pf_out.reserve(nout);
  s.pf_e.clear();
  s.pf_e.reserve(nterm);
  s.pf_w.clear();
  s.pf_w.reserve(nterm);
  for (int task = 0; task < ntask; ++task) {
    const int base = (int)s.pf_e.size();
    for (PfOut o : outs[task]) {
      o.beg += base;
      s.pf_out.push_back(o);
    }
    s.pf_e.insert(s.pf_e.end(), es[task].begin(), es[task].end());
    s.pf_w.insert(s.pf_w.end(), ws[task].begin(), ws[task].end());
  }
}

Space* build_space(int emax, const std::vector<int>& n, const std::vector<int>& l, const std::vector<int>& j2,
                   const std::vector<int>& tz2, const std::vector<double>& occ)
{
  Space* sp = new Space();
  Space& s = *sp;
  s.emax = emax;
  s.norb = (int)n.size();
  s.n = n; s.l = l; s.j2 = j2; s.tz2 = tz2; s.occ = occ;
  int j2max = 0;
  for (int i = 0; i < s.norb; ++i) {
    if (j2[i] < 1 || !(j2[i] & 1) || (tz2[i] != 1 && tz2[i] != -1) || l[i] < 0)
      throw std::runtime_error("invalid orbit quantum numbers");
    if (j2[i] > 2 * emax + 1) throw std::runtime_error("orbit j exceeds 2*emax+1");
    j2max = std::max(j2max, j2[i]);
    if (occ[i] >= OCC_CUT) s.holes.push_back(i);
  }
  if (j2max > 63) throw std::runtime_error("orbit j2 above 63 is not supported");
  s.NJ = j2max + 1;
  s.nch = 6 * (j2max + 1);  // ModelSpace::AddOrbit, src/ModelSpace.cc:936-946
  s.nkets = s.norb * (s.norb + 1) / 2;

  // one-body channels (l, j2, tz2)
  s.ob_start.resize(s.norb);
  s.ob_count.resize(s.norb);
  for (int i = 0; i < s.norb; ++i) {
    s.ob_start[i] = (int)s.ob_list.size();
    for (int a = 0; a < s.norb; ++a)
      if (l[a] == l[i] && j2[a] == j2[i] && tz2[a] == tz2[i]) s.ob_list.push_back(a);
    s.ob_count[i] = (int)s.ob_list.size() - s.ob_start[i];
  }

  // channels
  s.ch.resize(s.nch);
  s.cc.resize(s.nch);
  s.ketJ_loc.assign((size_t)s.nkets * s.NJ, -1);
  s.ccJ_loc.assign((size_t)s.nkets * s.NJ, -1);
  for (int c = 0; c < s.nch; ++c) {
    int J = c / 6, Tz = (c % 6) / 2 - 1, par = c % 2;
    Chan& C = s.ch[c];
    Chan& K = s.cc[c];
    C.J = K.J = J;
    C.parity = K.parity = par;
    C.Tz = K.Tz = Tz;
    for (int p = 0; p < s.norb; ++p)
      for (int q = p; q < s.norb; ++q) {
        if ((l[p] + l[q]) % 2 != par) continue;
        if (j2[p] + j2[q] < 2 * J) continue;
        if (std::abs(j2[p] - j2[q]) > 2 * J) continue;
        int k = ket_index(s.norb, p, q);
        bool hp = occ[p] > OCC_CUT, hq = occ[q] > OCC_CUT;
        bool lp = occ[p] < OCC_CUT, lq = occ[q] < OCC_CUT;
        if (!(p == q && J % 2 != 0) && tz2[p] + tz2[q] == 2 * Tz) {
          int loc = C.n();
          s.ketJ_loc[(size_t)J * s.nkets + k] = loc;
          C.p.push_back(p);
          C.q.push_back(q);
          if (lp && lq) C.pp.push_back(loc);
          if (hp != hq) C.ph.push_back(loc);
          if (hp && hq) C.hh.push_back(loc);
        }
        if (std::abs(tz2[p] - tz2[q]) == 2 * Tz) {
          int loc = K.n();
          s.ccJ_loc[(size_t)J * s.nkets + k] = loc;
          K.p.push_back(p);
          K.q.push_back(q);
          if (lp && lq) K.pp.push_back(loc);
          if (hp != hq) K.ph.push_back(loc);
          if (hp && hq) K.hh.push_back(loc);
        }
      }
  }

  // arena layout
  int64_t cur = round32(32 + (int64_t)s.norb * s.norb);
  for (int c = 0; c < s.nch; ++c) {
    s.ch[c].off = cur;
    cur = round32(cur + (int64_t)s.ch[c].n() * s.ch[c].n());
  }
  s.arena = cur;

  build_sixj_table(s);

  // ---- ladder work lists: w = (pp: 1) + (hh: nbar nbar - n n) + (ph: nbar nbar)
  //      (ConstructScalarMpp_Mhh, src/Commutator.cc:1170-1183, Mpp - Mhh)
  s.ladder_kidx_off.assign(s.nch, -1);
  s.ladder_w_off.assign(s.nch, -1);
  for (int c = 0; c < s.nch; ++c) {
    const Chan& C = s.ch[c];
    if (C.n() == 0) continue;
    std::vector<std::pair<int, double>> kw;
    for (int i = 0; i < C.n(); ++i) {
      double op = occ[C.p[i]], oq = occ[C.q[i]];
      double w = 0;
      bool hp = op > OCC_CUT, hq = oq > OCC_CUT, lp = op < OCC_CUT, lq = oq < OCC_CUT;
      if (lp && lq) w += 1.0;
      if (hp && hq) w += (1 - op) * (1 - oq) - op * oq;
      if (hp != hq) w += (1 - op) * (1 - oq);
      if (w != 0.0) kw.push_back({i, w});
    }
    if (kw.empty()) continue;
    s.ladder_kidx_off[c] = (int)s.kidx.size();
    s.ladder_w_off[c] = (int)s.kweight.size();
    for (auto& x : kw) {
      s.kidx.push_back(x.first);
      s.kweight.push_back(x.second);
    }
    SymGemmJob jb;
    jb.a_off = C.off;
    jb.b_off = C.off;
    jb.out_off = C.off;
    jb.m = C.n();
    jb.K = (int)kw.size();
    jb.lda = jb.ldb = jb.ldo = C.n();
    jb.kidx_off = s.ladder_kidx_off[c];
    jb.w_off = s.ladder_w_off[c];
    s.ladder_jobs.push_back(jb);
  }

  // ---- Pandya work lists (DoPandyaTransformation_SingleChannel_XandY, src/Commutator.cc:1392-1485)
  s.cc_nph.assign(s.nch, 0);
  s.cc_ph_off.assign(s.nch, 0);
  s.xb_off.assign(s.nch, 0);
  s.zb_off.assign(s.nch, 0);
  s.cc_phase_off.assign(s.nch, 0);
  int64_t xb = 0, zb = 0;
  for (int c = 0; c < s.nch; ++c) {
    const Chan& K = s.cc[c];
    s.cc_ph_off[c] = (int)s.cc_ph.size();
    for (int x : K.hh) s.cc_ph.push_back(x);
    for (int x : K.ph) s.cc_ph.push_back(x);
    s.cc_nph[c] = (int)(K.hh.size() + K.ph.size());
    s.cc_phase_off[c] = (int)s.phase_tab.size();
    for (int i = 0; i < K.n(); ++i) s.phase_tab.push_back(iphase((j2[K.p[i]] + j2[K.q[i]]) / 2));
    s.xb_off[c] = xb;
    s.zb_off[c] = zb;
    int ncc = K.n();
    int K2 = 2 * s.cc_nph[c];
    xb = round32(xb + (int64_t)ncc * K2);
    zb = round32(zb + (int64_t)ncc * 2 * ncc);
    if (ncc == 0 || K2 == 0) continue;
    SymGemmJob head;
    head.a_off = s.xb_off[c];
    head.b_off = s.xb_off[c];
    head.out_off = s.zb_off[c];
    head.m = ncc;
    head.K = K2;
    head.lda = head.ldb = head.ldo = ncc;
    SymGemmJob tail = head;
    tail.out_off = s.zb_off[c] + (int64_t)ncc * ncc;
    tail.phase_off = s.cc_phase_off[c];
    s.zbar_jobs.push_back(head);
    s.zbar_jobs.push_back(tail);
  }
  s.xb_total = xb;
  s.zb_total = zb;
  build_pandya_fwd(s);

  // ---- small-term work lists
  s.hh_off.assign(s.nch + 1, 0);
  for (int c = 0; c < s.nch; ++c) {
    const Chan& C = s.ch[c];
    int J = C.J;
    (void)J;
    s.hh_off[c] = (int)s.hh_list.size();
    for (int x : C.hh) s.hh_list.push_back(x);
    for (int i = 0; i < C.n(); ++i) {
      double op = occ[C.p[i]], oq = occ[C.q[i]];
      bool hp = op > OCC_CUT, hq = oq > OCC_CUT, lp = op < OCC_CUT, lq = oq < OCC_CUT;
      double wpp = 0, wnn = 0;
      if (lp && lq) wpp = 1.0;  // pp rows enter unweighted (src/Commutator.cc:1176, :619)
      if (hp && hq) {
        wpp = (1 - op) * (1 - oq);
        wnn = op * oq;
      }
      if (hp != hq) wpp = (1 - op) * (1 - oq);
      s.ket_wpp.push_back(wpp);
      s.ket_nn.push_back(wnn);
    }
    for (int x : C.hh) {
      s.items220.push_back(c);
      s.items220.push_back(x);
    }
  }
  s.hh_off[s.nch] = (int)s.hh_list.size();
  for (int i = 0; i < s.norb; ++i)
    for (int k = 0; k < s.ob_count[i]; ++k) {
      int j = s.ob_list[s.ob_start[i] + k];
      if (j < i) continue;
      s.pairs1b.push_back(i);
      s.pairs1b.push_back(j);
      for (int c = 0; c < s.norb; ++c) {
        s.items221.push_back(i);
        s.items221.push_back(j);
        s.items221.push_back(c);
      }
    }
  // comm122ss gathers (src/Commutator.cc:862-903)
  const double SQ2 = 1.4142135623730950488;
  for (int c = 0; c < s.nch; ++c) {
    const Chan& C = s.ch[c];
    int J = C.J;
    for (int ij = 0; ij < C.n(); ++ij) {
      int i = C.p[ij], j = C.q[ij];
      int flip = -iphase((j2[i] + j2[j]) / 2 - J);
      int first = (int)s.it122_loc.size();
      for (int k = 0; k < s.ob_count[i]; ++k) {
        int a = s.ob_list[s.ob_start[i] + k];
        int loc = s.ketJ_loc[(size_t)J * s.nkets + ket_index(s.norb, std::min(a, j), std::max(a, j))];
        if (loc < 0) continue;
        double f = a > j ? flip : (a == j ? SQ2 : 1.0);
        if (i == j) f = f / SQ2 * 2.0;
        s.it122_loc.push_back(loc);
        s.it122_a.push_back(a);
        s.it122_src.push_back(i);
        s.it122_f.push_back(f);
      }
      if (i != j)
        for (int k = 0; k < s.ob_count[j]; ++k) {
          int a = s.ob_list[s.ob_start[j] + k];
          int loc = s.ketJ_loc[(size_t)J * s.nkets + ket_index(s.norb, std::min(a, i), std::max(a, i))];
          if (loc < 0) continue;
          double f = i > a ? flip : (i == a ? SQ2 : 1.0);
          s.it122_loc.push_back(loc);
          s.it122_a.push_back(a);
          s.it122_src.push_back(j);
          s.it122_f.push_back(f);
        }
      s.cols122.push_back(c);
      s.cols122.push_back(ij);
      s.cols122.push_back(first);
      s.cols122.push_back((int)s.it122_loc.size() - first);
    }
  }
  return sp;
}

template <class T>
static T* dev_copy(Space& s, const std::vector<T>& v)
{
  void* p = nullptr;
  size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
  if (cudaMalloc(&p, bytes) != cudaSuccess) throw std::runtime_error("cudaMalloc failed for space tables");
  s.dev_allocs.push_back(p);
  if (!v.empty() && cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    throw std::runtime_error("cudaMemcpy failed for space tables");
  return (T*)p;
}

void upload_space(Space& s)
{
  DevSpace& d = s.dev;
  d.norb = s.norb;
  d.nch = s.nch;
  d.nkets = s.nkets;
  d.NJ = s.NJ;
  d.d1 = s.d1;
  d.l = dev_copy(s, s.l);
  d.j2 = dev_copy(s, s.j2);
  d.tz2 = dev_copy(s, s.tz2);
  d.occ = dev_copy(s, s.occ);
  d.ob_start = dev_copy(s, s.ob_start);
  d.ob_count = dev_copy(s, s.ob_count);
  d.ob_list = dev_copy(s, s.ob_list);
  d.ketJ_loc = dev_copy(s, s.ketJ_loc);
  d.ccJ_loc = dev_copy(s, s.ccJ_loc);
  std::vector<int> ch_n(s.nch), ch_kofs(s.nch), kp, kq, cc_n(s.nch), cc_kofs(s.nch), cp, cq;
  std::vector<long long> ch_off(s.nch);
  for (int c = 0; c < s.nch; ++c) {
    ch_n[c] = s.ch[c].n();
    ch_off[c] = s.ch[c].off;
    ch_kofs[c] = (int)kp.size();
    kp.insert(kp.end(), s.ch[c].p.begin(), s.ch[c].p.end());
    kq.insert(kq.end(), s.ch[c].q.begin(), s.ch[c].q.end());
    cc_n[c] = s.cc[c].n();
    cc_kofs[c] = (int)cp.size();
    cp.insert(cp.end(), s.cc[c].p.begin(), s.cc[c].p.end());
    cq.insert(cq.end(), s.cc[c].q.begin(), s.cc[c].q.end());
  }
  d.ch_n = dev_copy(s, ch_n);
  d.ch_off = dev_copy(s, ch_off);
  d.ch_kofs = dev_copy(s, ch_kofs);
  d.ket_p = dev_copy(s, kp);
  d.ket_q = dev_copy(s, kq);
  d.cc_n = dev_copy(s, cc_n);
  d.cc_kofs = dev_copy(s, cc_kofs);
  d.cc_p = dev_copy(s, cp);
  d.cc_q = dev_copy(s, cq);
  d.sixj_base = dev_copy(s, s.sixj_base);
  d.sixj_val = dev_copy(s, s.sixj_val);
  d.sixj_wval = dev_copy(s, s.sixj_wval);
  d.sixj_wf = dev_copy(s, s.sixj_wf);

  DevWork& w = s.work;
  w.ket_wpp = dev_copy(s, s.ket_wpp);
  w.ket_nn = dev_copy(s, s.ket_nn);
  w.hh_off = dev_copy(s, s.hh_off);
  w.hh_list = dev_copy(s, s.hh_list);
  w.items220 = dev_copy(s, s.items220);
  w.n220 = (int)s.items220.size() / 2;
  w.pairs1b = dev_copy(s, s.pairs1b);
  w.npairs1b = (int)s.pairs1b.size() / 2;
  w.items221 = dev_copy(s, s.items221);
  w.n221 = (int)s.items221.size() / 3;
  w.cols122 = dev_copy(s, s.cols122);
  w.ncols122 = (int)s.cols122.size() / 4;
  w.it122_loc = dev_copy(s, s.it122_loc);
  w.it122_a = dev_copy(s, s.it122_a);
  w.it122_src = dev_copy(s, s.it122_src);
  w.it122_f = dev_copy(s, s.it122_f);
  w.kidx = dev_copy(s, s.kidx);
  w.kweight = dev_copy(s, s.kweight);
  w.phase_tab = dev_copy(s, s.phase_tab);
  w.cc_nph = dev_copy(s, s.cc_nph);
  w.cc_ph_off = dev_copy(s, s.cc_ph_off);
  w.cc_ph = dev_copy(s, s.cc_ph);
  std::vector<long long> xo(s.xb_off.begin(), s.xb_off.end()), zo(s.zb_off.begin(), s.zb_off.end());
  w.xb_off = dev_copy(s, xo);
  w.zb_off = dev_copy(s, zo);
  w.cc_phase_off = dev_copy(s, s.cc_phase_off);
  w.pf_out = dev_copy(s, s.pf_out);
  w.n_pfout = (int)s.pf_out.size();
  w.pf_e = dev_copy(s, s.pf_e);
  w.pf_w = dev_copy(s, s.pf_w);
  std::vector<float2> wf(s.pf_w.size());
  for (size_t k = 0; k < wf.size(); ++k) {
    const float hi = (float)s.pf_w[k];
    wf[k] = make_float2(hi, (float)(s.pf_w[k] - (double)hi));
  }
  w.pf_wf = dev_copy(s, wf);
}

// Blocks of the quadruple-ordered inverse Pandya transform (split form).
// Orbits fall into four classes by (parity, Tz).  For a bra orbit i, a ket
// orbit k >= i and the class of j, the class of l is fixed by parity and Tz
// conservation, and every quadruple (i, j, k, l) of that (i, k, class) has its
// Z elements in one rectangle per channel J: rows (i, j), columns (k, l),
// consecutive kets in the channel's order.  A block takes such an (i, k, class)
// group, or a run of its j rows when the group's Zbar values and results would
// not fit in `budget` bytes of shared memory.
void build_invq_tasks(Space& s, int budget)
{
  const int N = s.norb;
  s.cls_list.clear();
  s.cls_off.assign(5, 0);
  s.invq_tasks.clear();
  s.invq_smem = 0;
  bool fits = s.NJ < kInvqMaxJ;  // J' and J counts < 32: 5-bit fields
  for (int c = 0; c < 4; ++c) {
    s.cls_off[c] = (int)s.cls_list.size();
    for (int o = 0; o < N; ++o)
      if (((s.l[o] & 1) | (s.tz2[o] > 0 ? 2 : 0)) == c) s.cls_list.push_back(o);
    if ((int)s.cls_list.size() - s.cls_off[c] > kInvqMaxOrb) fits = false;
  }
  s.cls_off[4] = (int)s.cls_list.size();
  s.cls_sort.assign(s.cls_list.size(), 0);
  for (int c = 0; c < 4; ++c) {
    std::vector<int> pos;
    for (int x = 0; x < s.cls_off[c + 1] - s.cls_off[c]; ++x) pos.push_back(x);
    const int* o = s.cls_list.data() + s.cls_off[c];
    std::stable_sort(pos.begin(), pos.end(), [&](int a, int b) { return s.j2[o[a]] < s.j2[o[b]]; });
    for (size_t x = 0; x < pos.size(); ++x) s.cls_sort[s.cls_off[c] + x] = (unsigned char)pos[x];
  }
  // beyond the block's table sizes (emax > 14 for a full space) the split form
  // keeps the channel-tiled kernel: no blocks
  if (!fits) return;
  auto emit = [&](int i, int k, int cj, int cl, int jf, int jn, int lf, int ln, int slots) {
    s.invq_tasks.push_back(i | (k << 16));
    s.invq_tasks.push_back(cj | (cl << 8));
    s.invq_tasks.push_back(jf | (jn << 16));
    s.invq_tasks.push_back(lf | (ln << 16));
    s.invq_smem = std::max(s.invq_smem, invq_block_bytes(jn, ln, slots));
  };
  for (int i = 0; i < N; ++i)
    for (int k = i; k < N; ++k)
      for (int cj = 0; cj < 4; ++cj) {
        int pj = cj & 1, tzj = (cj & 2) ? 1 : -1;
        int tzl = s.tz2[i] + tzj - s.tz2[k];
        if (tzl != 1 && tzl != -1) continue;
        int cl = ((s.l[i] + pj + s.l[k]) & 1) | (tzl > 0 ? 2 : 0);
        const int* Jc = s.cls_list.data() + s.cls_off[cj];
        const int* Lc = s.cls_list.data() + s.cls_off[cl];
        int nJc = s.cls_off[cj + 1] - s.cls_off[cj], nLc = s.cls_off[cl + 1] - s.cls_off[cl];
        int jf = (int)(std::lower_bound(Jc, Jc + nJc, i) - Jc);
        int lf = (int)(std::lower_bound(Lc, Lc + nLc, k) - Lc);
        int jtot = nJc - jf, ln = nLc - lf;
        if (jtot <= 0 || ln <= 0) continue;
        int r0 = 0, slots = 0;
        bool any = false;
        for (int r = 0; r < jtot; ++r) {
          int j = Jc[jf + r];
          int rs = 0;
          bool ra = false;
          for (int x = 0; x < ln; ++x) {
            int l = Lc[lf + x];
            int n1, n2, nJ, Jlo, lo1, lo2;
            if (invq_counts(i, j, k, l, s.j2[i], s.j2[j], s.j2[k], s.j2[l], 1, n1, n2, nJ, Jlo, lo1, lo2)) {
              rs += invq_slot_bytes(n1, n2, nJ);
              ra = true;
            }
          }
          if (r > r0 && invq_block_bytes(r - r0 + 1, ln, slots + rs) > budget) {
            if (any) emit(i, k, cj, cl, jf + r0, r - r0, lf, ln, slots);
            r0 = r;
            slots = 0;
            any = false;
          }
          slots += rs;
          any = any || ra;
        }
        if (any) emit(i, k, cj, cl, jf + r0, jtot - r0, lf, ln, slots);
      }
  if (s.invq_smem > 160 * 1024) {
    s.invq_tasks.clear();
    s.invq_smem = 0;
  }
}

Space::~Space()
{
  for (auto& kv : tensors) delete kv.second;
  for (void* p : dev_allocs) cudaFree(p);
  for (Scratch* sc : {&s_xb, &s_yb, &s_yf, &s_zb, &s_w2, &s_red, &s_split_a, &s_split_b, &s_split_e, &s_jobs})
    if (sc->ptr) cudaFree(sc->ptr);
}

}  // namespace imsrg
