// Inverse Pandya transform from precomputed descriptors.
//
// AddInversePandyaTransformation (src/Commutator.cc:1501-1616) adds to every
// upper-triangle element Z_J(ij, kl) (and its mirror) two J' sums over Zbar:
//     A1 = sum_J' (2J'+1) {j_i j_j J; j_k j_l J'} Zbar_J'(il, kj)
//     A2 = sum_J' (2J'+1) {j_j j_i J; j_k j_l J'} Zbar_J'(ik, lj)
// For one orbit quadruple (i, j, k, l) both sums read the same Zbar values in
// every channel J the quadruple lives in; only the 6j weights change with J.
//
// Everything about that computation except the values is a property of the
// model space: which Zbar elements a quadruple reads, which 6j row weighs them
// for each J, which Z elements receive the result, with what sign and norm.
// So it is worked out once per space, on the host (build_invd), into flat
// descriptor arrays, and the kernel does nothing per call but loads and FMAs:
//   1. a block stages its quadruples' Zbar values in shared memory (a thread
//      per value; the Zbar element index of each is precomputed, int32);
//   2. a thread per result (quadruple, J) reads a 24-byte descriptor: offsets
//      of its staged values and counts, the 6j weight rows, its two Z element
//      indices, and a few bits for the combination
//        z = scale * (c1 A1 + c2 A2),  c1 in {0, 1, 2},  c2 in {0, +-1, +-hZ},
//      then Z(ij, kl) += z and Z(kl, ij) += hZ z.
// Only the upper triangle of each Zbar block is read: Zbar is symmetric by
// construction (head: Zbar(r, c) = hZ Zbar(c, r); tail: Zbar(r, n + c) =
// phi_r phi_c Zbar(c, n + r), phi of a ket (p, q) = (-1)^((j_p + j_q) / 2)), so
// a lower-triangle value is read from its mirror with that sign, and the Zbar
// product can skip the mirror half of its stores.
// Quadruples are enumerated by (i, k, parity/Tz class of j, j, l), so blocks
// running together read neighbouring Zbar columns and write neighbouring Z
// rectangles.  The sums run in FP64 (DF = false) or in double-float on the
// FP32 pipe (DF = true: Zbar values and weights as (hi, lo) float pairs).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "dfloat.cuh"
#include "kernels.cuh"
#include "prof.hpp"
#include "space.hpp"

namespace imsrg {

namespace {

// descriptor bit fields (second int2 word pair), see build_invd
constexpr int kNShift = 16;     // n1 / n2: bits 16..20
constexpr int kCShift = 21;     // c1 code (0, 1, 2) / c2 code (0, +1, -1): bits 21..22
constexpr int kFShift = 23;     // x: scale code (0: 1, 1: 1/2, 2: 1/sqrt2); y: c2 times hZ
constexpr int kDiagBit = 25;    // x: diagonal element, skipped for an anti-hermitian Z
constexpr int kThreads = 256;
// staged value: Zbar element index in bits 0..28; bit 29 negates the value,
// bit 30 multiplies it by hZ (an element of the lower triangle read as its
// mirror in the upper one)
constexpr int kIdxMask = (1 << 29) - 1;
constexpr int kNegBit = 29;
constexpr int kHzBit = 30;

}  // namespace

// ------------------------------------------------------------------- host
namespace {

// the blocks of the quadruples with first orbit i (block offsets relative to
// this part), in (k, class of j, j, l) order, j and l by (2j, orbit)
void build_invd_part(const Space& s, int i, const std::vector<int> (&cls)[4], InvdPlan& out, int stage_max,
                     int res_max, bool stage_weights)
{
  const int N = s.norb, nk = s.nkets;
  const int d1 = s.d1;
  struct Res {
    int4 a;
    int2 b;
    int cost;
  };
  std::vector<Res> res;
  std::vector<int> stage;
  // the block's 6j weight rows: first global weight index -> row length
  std::map<int, int> wrows;
  int nweights = 0;
  auto flush = [&]() {
    if (res.empty()) {
      stage.clear();
      wrows.clear();
      nweights = 0;
      return;
    }
    // weight rows staged in shared memory after the Zbar values; results
    // refer to them by their offset there
    const int wbase = (int)out.wrow.size();
    int nw = 0;
    if (stage_weights) {
      std::map<int, int> woff;
      for (auto& r : wrows) {
        woff[r.first] = nw;
        out.wrow.push_back(make_int2(r.first, nw | (r.second << 20)));
        nw += r.second;
      }
      for (Res& r : res) {
        if ((r.b.x >> kCShift) & 3) r.a.x = woff.at(r.a.x);
        if ((r.b.y >> kCShift) & 3) r.a.y = woff.at(r.a.y);
      }
    }
    // results in 6j weight-row order (then output order): the lanes of a
    // warp then read the same weight rows, one L1 wavefront where output
    // order gave up to 32 (0.76 -> 0.72 ms at emax=10; the Z updates they
    // scatter are two loads and two stores a result)
    std::stable_sort(res.begin(), res.end(), [](const Res& x, const Res& y) {
      if (x.a.x != y.a.x) return x.a.x < y.a.x;
      if (x.a.y != y.a.y) return x.a.y < y.a.y;
      return x.a.z < y.a.z;
    });
    // staged values loaded in address order, each to its slot
    std::vector<int> ord(stage.size());
    for (size_t e = 0; e < ord.size(); ++e) ord[e] = (int)e;
    std::stable_sort(ord.begin(), ord.end(),
                     [&](int x, int y) { return (stage[x] & kIdxMask) < (stage[y] & kIdxMask); });
    out.blocks.push_back(make_int4((int)out.sidx.size(), (int)stage.size(), (int)out.dA.size(), (int)res.size()));
    out.wblk.push_back(make_int2(wbase, (int)out.wrow.size() - wbase));
    out.stage_max = std::max(out.stage_max, (int)stage.size() + nw);
    for (int e : ord) {
      out.sidx.push_back(stage[e]);
      out.sslot.push_back((unsigned short)e);
    }
    for (const Res& r : res) {
      out.dA.push_back(r.a);
      out.dB.push_back(r.b);
    }
    res.clear();
    stage.clear();
    wrows.clear();
    nweights = 0;
  };
  auto cc_of = [&](int J, int a, int b) { return chan_index(J, (s.l[a] + s.l[b]) & 1, std::abs(s.tz2[a] - s.tz2[b]) / 2); };
  // the staged word of Zbar element (row r, column col) of CC channel cc:
  // lower-triangle elements of the head and tail blocks from their mirrors
  auto zword = [&](int cc, int r, int col) {
    const int ncc = s.cc[cc].n();
    const bool tail = col >= ncc;
    int c = tail ? col - ncc : col;
    int flags = 0;
    if (r > c) {
      if (tail) {
        const int* phi = s.phase_tab.data() + s.cc_phase_off[cc];
        if (phi[r] * phi[c] < 0) flags |= 1 << kNegBit;
      } else {
        flags |= 1 << kHzBit;
      }
      std::swap(r, c);
    }
    const long long e = s.zb_off[cc] + (long long)(tail ? c + ncc : c) * ncc + r;
    return (int)e | flags;
  };
  std::vector<Res> pres;
  std::vector<int> pst;
  {
    for (int k = i; k < N; ++k)
      for (int cj = 0; cj < 4; ++cj) {
        const int pj = cj & 1, tzj = (cj & 2) ? 1 : -1;
        const int tzl = s.tz2[i] + tzj - s.tz2[k];
        if (tzl != 1 && tzl != -1) continue;
        const int cl = ((s.l[i] + pj + s.l[k]) & 1) | (tzl > 0 ? 2 : 0);
        for (int j : cls[cj]) {
          if (j < i) continue;
          for (int l : cls[cl]) {
            if (l < k) continue;
            const int ji = s.j2[i], jj = s.j2[j], jk = s.j2[k], jl = s.j2[l];
            int n1, n2, nJ, Jlo, lo1, lo2;
            if (!invq_counts(i, j, k, l, ji, jj, jk, jl, 1, n1, n2, nJ, Jlo, lo1, lo2)) continue;
            const bool ev = (i == j) || (k == l);
            const int a6 = (ji - 1) >> 1, b6 = (jj - 1) >> 1, c6 = (jk - 1) >> 1, e6 = (jl - 1) >> 1;
            const int J3min = std::abs(ji - jj) >> 1;
            const int base1 = s.sixj_base[((a6 * d1 + b6) * d1 + c6) * d1 + e6];
            const int base2 = s.sixj_base[((b6 * d1 + a6) * d1 + c6) * d1 + e6];
            const int ph4 = iphase((ji + jj + jk + jl) / 2);
            const int chJ_par = (s.l[i] + s.l[j]) & 1, chJ_tz = (s.tz2[i] + s.tz2[j]) / 2;
            pres.clear();
            for (int t = 0; t < nJ; ++t) {
              const int J = Jlo + (ev ? 2 * t : t);
              const int phJ = iphase((jk + jl) / 2 - J);
              int c1, c2 = 0, hzdep = 0;
              if (ev) {
                const int f = (k == l) ? phJ : phJ * ph4;
                c1 = f > 0 ? 0 : 2;
              } else {
                c1 = 1;
                // z = A1 - phJ tsign A2, tsign = ph4 (l > j) or hZ
                if (l > j) {
                  c2 = phJ * ph4 > 0 ? 2 : 1;  // code 2: -1, code 1: +1
                } else {
                  c2 = phJ > 0 ? 2 : 1;        // times hZ at run time
                  hzdep = 1;
                }
                if (n2 == 0) c2 = 0;
              }
              // an element whose sums vanish by symmetry still gets a result
              // (z = 0): every upper-triangle element of Z has exactly one, so
              // the kernel can also apply comm122ss's W2 + h_Z W2^T there
              if ((c1 == 0 || n1 == 0) && c2 == 0) c1 = 0;
              const int scale = (i == j && k == l) ? 1 : (ev ? 2 : 0);
              const int ib = s.ketJ_loc[(size_t)J * nk + ket_index(N, i, j)];
              const int ik = s.ketJ_loc[(size_t)J * nk + ket_index(N, k, l)];
              if (ib < 0 || ik < 0) throw std::runtime_error("inverse Pandya descriptors: missing ket");
              const Chan& C = s.ch[chan_index(J, chJ_par, chJ_tz)];
              const int n = C.n();
              const long long o1 = C.off + (long long)ik * n + ib;
              const long long o2 = ib != ik ? C.off + (long long)ib * n + ik : -1;
              Res r;
              r.a = make_int4(base1 + (J - J3min) * n1, n2 ? base2 + (J - J3min) * n2 : 0, (int)o1, (int)o2);
              // staged offsets are filled in when the pair joins a block
              r.b = make_int2((n1 << kNShift) | ((c1 == 0 ? 0 : c1) << kCShift) | (scale << kFShift) |
                                  ((i == k && j == l) ? 1 << kDiagBit : 0),
                              (n2 << kNShift) | (c2 << kCShift) | (hzdep << kFShift));
              r.cost = (c1 ? n1 : 0) + (c2 ? n2 : 0);
              pres.push_back(r);
            }
            if (pres.empty()) continue;
            // the pair's Zbar values: sum 1 then sum 2
            pst.clear();
            for (int x = 0; x < n1; ++x) {
              const int Jp = lo1 + x;
              const int cc = cc_of(Jp, i, l);
              const int ncc = s.cc[cc].n();
              const int il = s.ccJ_loc[(size_t)Jp * nk + ket_index(N, i, l)];
              const int kj0 = s.ccJ_loc[(size_t)Jp * nk + ket_index(N, std::min(k, j), std::max(k, j))];
              if (il < 0 || kj0 < 0) throw std::runtime_error("inverse Pandya descriptors: missing CC ket");
              pst.push_back(zword(cc, il, kj0 + (k > j ? ncc : 0)));
            }
            for (int x = 0; x < n2; ++x) {
              const int Jp = lo2 + x;
              const int cc = cc_of(Jp, i, k);
              const int ncc = s.cc[cc].n();
              const int cik = s.ccJ_loc[(size_t)Jp * nk + ket_index(N, i, k)];
              const int lj = s.ccJ_loc[(size_t)Jp * nk + ket_index(N, std::min(l, j), std::max(l, j))];
              if (cik < 0 || lj < 0) throw std::runtime_error("inverse Pandya descriptors: missing CC ket");
              pst.push_back(zword(cc, lj, cik + (l > j ? ncc : 0)));
            }
            // the weight rows this pair adds to the block
            int wnew = 0;
            for (const Res& r : pres) {
              if (((r.b.x >> kCShift) & 3) && !wrows.count(r.a.x)) wnew += n1;
              if (((r.b.y >> kCShift) & 3) && !wrows.count(r.a.y)) wnew += n2;
            }
            if (!stage_weights) wnew = 0;
            if ((int)(stage.size() + pst.size()) > stage_max || nweights + wnew > stage_max ||
                (int)(res.size() + pres.size()) > res_max) {
              flush();
              wnew = 0;
              std::map<int, int> fresh;
              for (const Res& r : pres) {
                if ((r.b.x >> kCShift) & 3) fresh[r.a.x] = n1;
                if ((r.b.y >> kCShift) & 3) fresh[r.a.y] = n2;
              }
              for (auto& f : fresh) wnew += f.second;
              if (!stage_weights) wnew = 0;
            }
            const int z1 = (int)stage.size(), z2 = z1 + n1;
            for (Res& r : pres) {
              r.b.x |= z1 & 0xFFFF;
              r.b.y |= z2 & 0xFFFF;
              if ((r.b.x >> kCShift) & 3) wrows[r.a.x] = n1;
              if ((r.b.y >> kCShift) & 3) wrows[r.a.y] = n2;
              res.push_back(r);
            }
            nweights += wnew;
            stage.insert(stage.end(), pst.begin(), pst.end());
          }
        }
        flush();  // a block never spans two (i, k, class) groups
      }
  }
  flush();
}

}  // namespace

void build_invd(const Space& s, InvdPlan& out, int stage_max, int res_max, bool stage_weights)
{
  const int N = s.norb;
  if (s.arena >= (1ll << 31) || s.zb_total > kIdxMask)
    throw std::runtime_error("inverse Pandya descriptors: arena or Zbar beyond their index fields");
  stage_max = std::max(64, std::min(stage_max, 8192));
  res_max = std::max(64, res_max);
  // orbits by (parity, Tz) class, ordered by (2j, orbit): quadruples that
  // follow each other share their 6j weight rows
  std::vector<int> cls[4];
  for (int o = 0; o < N; ++o) cls[(s.l[o] & 1) | (s.tz2[o] > 0 ? 2 : 0)].push_back(o);
  for (auto& c : cls)
    std::stable_sort(c.begin(), c.end(), [&](int a, int b) { return s.j2[a] < s.j2[b]; });
  // one part per first orbit, built in parallel, then joined in order
  std::vector<InvdPlan> parts(N);
  std::vector<std::string> errs(N);
#pragma omp parallel for schedule(dynamic, 1)
  for (int i = 0; i < N; ++i) {
    try {
      build_invd_part(s, i, cls, parts[i], stage_max, res_max, stage_weights);
    } catch (std::exception& e) {
      errs[i] = e.what();
    }
  }
  for (const std::string& e : errs)
    if (!e.empty()) throw std::runtime_error(e);
  size_t nb = 0, ns = 0, nr = 0;
  for (const InvdPlan& p : parts) {
    nb += p.blocks.size();
    ns += p.sidx.size();
    nr += p.dA.size();
  }
  size_t nwt = 0;
  for (const InvdPlan& p : parts) nwt += p.wrow.size();
  if (ns >= (1ull << 31) || nr >= (1ull << 31) || nwt >= (1ull << 31))
    throw std::runtime_error("inverse Pandya descriptors: too many");
  out = InvdPlan();
  out.blocks.reserve(nb);
  out.sidx.reserve(ns);
  out.dA.reserve(nr);
  out.dB.reserve(nr);
  out.stage_max = 0;
  for (InvdPlan& p : parts) {
    const int so = (int)out.sidx.size(), ro = (int)out.dA.size(), wo = (int)out.wrow.size();
    for (int4 b : p.blocks) out.blocks.push_back(make_int4(b.x + so, b.y, b.z + ro, b.w));
    for (int2 w : p.wblk) out.wblk.push_back(make_int2(w.x + wo, w.y));
    out.wrow.insert(out.wrow.end(), p.wrow.begin(), p.wrow.end());
    out.sslot.insert(out.sslot.end(), p.sslot.begin(), p.sslot.end());
    out.sidx.insert(out.sidx.end(), p.sidx.begin(), p.sidx.end());
    out.dA.insert(out.dA.end(), p.dA.begin(), p.dA.end());
    out.dB.insert(out.dB.end(), p.dB.begin(), p.dB.end());
    out.stage_max = std::max(out.stage_max, p.stage_max);
    p = InvdPlan();
  }
}

// ----------------------------------------------------------------- device
namespace {

// the value z one descriptor adds to Z(ij, kl) (and hZ z to Z(kl, ij))
template <bool DF, bool SW>
__device__ __forceinline__ double invd_value(const int4 a, const int2 b, int hZ, const unsigned char* smem, int nstage,
                                           const double* __restrict__ wval, const float2* __restrict__ wf)
{
  const int n1 = (b.x >> kNShift) & 31, n2 = (b.y >> kNShift) & 31;
  const int c1 = (b.x >> kCShift) & 3, c2c = (b.y >> kCShift) & 3;
  const int scode = (b.x >> kFShift) & 3;
  int c2 = c2c == 0 ? 0 : (c2c == 1 ? 1 : -1);
  if ((b.y >> kFShift) & 1) c2 *= hZ;
  const int z1 = b.x & 0xFFFF, z2 = b.y & 0xFFFF;
  double z;
  if (DF) {
    const float2* zs = (const float2*)smem;
    const float2* ws = SW ? zs + nstage : wf;
    float s1 = 0.f, e1 = 0.f, s1b = 0.f, e1b = 0.f;
    if (c1) {
      int x = 0;
      for (; x + 1 < n1; x += 2) {
        df_fma(ws[a.x + x], zs[z1 + x], s1, e1);
        df_fma(ws[a.x + x + 1], zs[z1 + x + 1], s1b, e1b);
      }
      if (x < n1) df_fma(ws[a.x + x], zs[z1 + x], s1, e1);
      df_add(s1, e1, s1b, e1b, s1, e1);
      if (c1 == 2) {
        s1 = __fmul_rn(s1, 2.f);
        e1 = __fmul_rn(e1, 2.f);
      }
    }
    float hi = s1, lo = e1;
    if (c2) {
      float s2 = 0.f, e2 = 0.f, s2b = 0.f, e2b = 0.f;
      int x = 0;
      for (; x + 1 < n2; x += 2) {
        df_fma(ws[a.y + x], zs[z2 + x], s2, e2);
        df_fma(ws[a.y + x + 1], zs[z2 + x + 1], s2b, e2b);
      }
      if (x < n2) df_fma(ws[a.y + x], zs[z2 + x], s2, e2);
      df_add(s2, e2, s2b, e2b, s2, e2);
      if (c2 < 0) {
        s2 = -s2;
        e2 = -e2;
      }
      df_add(s1, e1, s2, e2, hi, lo);
    }
    z = ff2d(hi, lo);
  } else {
    const double* zs = (const double*)smem;
    const double* ws = SW ? zs + nstage : wval;
    double s1 = 0.0, s2 = 0.0;
    if (c1) {
      for (int x = 0; x < n1; ++x) s1 = fma(ws[a.x + x], zs[z1 + x], s1);
      if (c1 == 2) s1 *= 2.0;
    }
    if (c2) {
      for (int x = 0; x < n2; ++x) s2 = fma(ws[a.y + x], zs[z2 + x], s2);
      s1 = c2 > 0 ? s1 + s2 : s1 - s2;
    }
    z = s1;
  }
  if (scode == 1)
    z *= 0.5;
  else if (scode == 2)
    z *= 0.70710678118654752440;
  return z;
}

template <bool DF, bool SW, int R>
__global__ void __launch_bounds__(kThreads) k_pandya_inv_desc(const int4* __restrict__ blocks,
                                                              const int2* __restrict__ wblk,
                                                              const int2* __restrict__ wrow,
                                                              const int* __restrict__ sidx,
                                                              const unsigned short* __restrict__ sslot,
                                                              const int4* __restrict__ dA,
                                                              const int2* __restrict__ dB,
                                                              const double* __restrict__ wval,
                                                              const float2* __restrict__ wf,
                                                              const double* __restrict__ Zb, double* __restrict__ Z,
                                                              int hZ, const long long* __restrict__ zo,
                                                              const void* __restrict__ W2, int w2mode)
{
  if (zo) {
    Zb = (const double*)((const char*)Zb + zo[blockIdx.z * kZRoles + ZR_ZB]);
    Z = (double*)((char*)Z + zo[blockIdx.z * kZRoles + ZR_Z]);
  }
  extern __shared__ __align__(16) unsigned char smem[];
  const int4 bk = blocks[blockIdx.x];
  const int2 wb = wblk[blockIdx.x];
  const int tid = threadIdx.x;
  // 1. staging: the block's 6j weight rows, then its Zbar values (in address
  //    order, each to its slot), eight loads in flight per thread
  for (int r = tid; SW && r < wb.y; r += kThreads) {
    const int2 row = __ldg(wrow + wb.x + r);
    const int o = bk.y + (row.y & 0xFFFFF), n = row.y >> 20;
    for (int x = 0; x < n; ++x) {
      if (DF)
        ((float2*)smem)[o + x] = __ldg(wf + row.x + x);
      else
        ((double*)smem)[o + x] = __ldg(wval + row.x + x);
    }
  }
  {
    const int* si = sidx + bk.x;
    const unsigned short* sl = sslot + bk.x;
    for (int e0 = tid; e0 < bk.y; e0 += 8 * kThreads) {
      double v[8];
      int w[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + u * kThreads;
        w[u] = e < bk.y ? __ldg(si + e) : 0;
        v[u] = e < bk.y ? __ldg(Zb + (w[u] & kIdxMask)) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int e = e0 + u * kThreads;
        const bool neg = ((w[u] >> kNegBit) & 1) != (((w[u] >> kHzBit) & 1) && hZ < 0);
        if (neg) v[u] = -v[u];
        if (e < bk.y) {
          const int slot = __ldg(sl + e);
          if (DF)
            ((float2*)smem)[slot] = d2ff(v[u]);
          else
            ((double*)smem)[slot] = v[u];
        }
      }
    }
  }
  __syncthreads();
  // 2. a thread per result, R results in flight per thread: descriptors,
  //    then the old Z values, then the sums and the updates
  for (int e0 = tid; e0 < bk.w; e0 += R * kThreads) {
    int4 a[R];
    int2 b[R];
    double o1[R], o2[R];
    bool ok[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      const int e = e0 + u * kThreads;
      ok[u] = e < bk.w;
      if (ok[u]) {
        a[u] = __ldg(dA + bk.z + e);
        b[u] = __ldg(dB + bk.z + e);
        ok[u] = !(((b[u].x >> kDiagBit) & 1) && hZ < 0);
      }
    }
    // comm122ss's Z -= W2 + h_Z W2^T at the same two elements, when the
    // commutator folds it in here (w2mode 1: W2 as (hi, lo) float pairs,
    // 2: FP64); W2 has Z's layout
    double w1[R], w2[R];
#pragma unroll
    for (int u = 0; u < R; ++u) {
      w1[u] = 0.0;
      w2[u] = 0.0;
      if (ok[u]) {
        o1[u] = Z[a[u].z];
        o2[u] = a[u].w >= 0 ? Z[a[u].w] : 0.0;
        const int q = a[u].w >= 0 ? a[u].w : a[u].z;
        if (w2mode == 2) {
          const double wp = __ldg((const double*)W2 + a[u].z), wq = __ldg((const double*)W2 + q);
          w1[u] = wp + hZ * wq;
          w2[u] = wq + hZ * wp;
        } else if (w2mode == 1) {
          const float2 wp = __ldg((const float2*)W2 + a[u].z), wq = __ldg((const float2*)W2 + q);
          const float sg = hZ < 0 ? -1.f : 1.f;
          float hi, lo;
          df_add(wp.x, wp.y, sg * wq.x, sg * wq.y, hi, lo);
          w1[u] = ff2d(hi, lo);
          df_add(wq.x, wq.y, sg * wp.x, sg * wp.y, hi, lo);
          w2[u] = ff2d(hi, lo);
        }
      }
    }
#pragma unroll
    for (int u = 0; u < R; ++u) {
      if (!ok[u]) continue;
      const double z = invd_value<DF, SW>(a[u], b[u], hZ, smem, bk.y, wval, wf);
      Z[a[u].z] = w2mode ? (o1[u] + z) - w1[u] : o1[u] + z;
      if (a[u].w >= 0) Z[a[u].w] = w2mode ? (o2[u] + (hZ > 0 ? z : -z)) - w2[u] : o2[u] + (hZ > 0 ? z : -z);
    }
  }
}

}  // namespace

cudaError_t launch_pandya_inv_desc(const Space& s, const InvdDev& d, bool df, const double* Zb, double* Z, int hZ,
                                   cudaStream_t st, const long long* zo, int nz, const void* W2, int w2mode)
{
  if (w2mode && (zo || !d.covers_all)) return cudaErrorInvalidValue;
  if (d.nblocks == 0) return cudaSuccess;
  const size_t smem = (size_t)d.stage_max * 8;
  using Kern = void (*)(const int4*, const int2*, const int2*, const int*, const unsigned short*, const int4*,
                       const int2*, const double*, const float2*, const double*, double*, int, const long long*,
                       const void*, int);
  // [df][staged weights][results in flight: 1, 2, 4]
  static const Kern kerns[2][2][3] = {
      {{k_pandya_inv_desc<false, false, 1>, k_pandya_inv_desc<false, false, 2>, k_pandya_inv_desc<false, false, 4>},
       {k_pandya_inv_desc<false, true, 1>, k_pandya_inv_desc<false, true, 2>, k_pandya_inv_desc<false, true, 4>}},
      {{k_pandya_inv_desc<true, false, 1>, k_pandya_inv_desc<true, false, 2>, k_pandya_inv_desc<true, false, 4>},
       {k_pandya_inv_desc<true, true, 1>, k_pandya_inv_desc<true, true, 2>, k_pandya_inv_desc<true, true, 4>}}};
  const int ri = d.ilp >= 4 ? 2 : (d.ilp >= 2 ? 1 : 0);
  Kern kern = kerns[df ? 1 : 0][d.staged_weights ? 1 : 0][ri];
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return e;
  kern<<<dim3(d.nblocks, 1, nz), kThreads, smem, st>>>(d.blocks, d.wblk, d.wrow, d.sidx, d.sslot, d.dA, d.dB,
                                                       s.dev.sixj_wval, s.dev.sixj_wf, Zb, Z, hZ, zo, W2, w2mode);
  count_launch();
  return cudaGetLastError();
}

}  // namespace imsrg
