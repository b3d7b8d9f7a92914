// Tensor-operator layouts and angular-momentum tables (see tensor.hpp).
#include "tensor.hpp"

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <stdexcept>

#include "kernels.cuh"
#include "space.hpp"

namespace imsrg {
namespace {

int64_t round32(int64_t x) { return (x + 31) / 32 * 32; }

bool triad2(int a, int b, int c)  // doubled arguments
{
  if ((a + b + c) & 1) return false;
  return c <= a + b && c >= std::abs(a - b);
}

// compact {h1 h2 I3; h4 h5 I6} table of extent d1 (the layout sixj_slot reads)
void build_compact(int d1, std::vector<int>& base, std::vector<double>& val)
{
  base.assign((size_t)d1 * d1 * d1 * d1, 0);
  size_t tot = 0;
  for (int a = 0; a < d1; ++a)
    for (int b = 0; b < d1; ++b)
      for (int c = 0; c < d1; ++c)
        for (int d = 0; d < d1; ++d) {
          int jj1 = 2 * a + 1, jj2 = 2 * b + 1, jj4 = 2 * c + 1, jj5 = 2 * d + 1;
          int n3 = (jj1 + jj2 - std::abs(jj1 - jj2)) / 2 + 1;
          int J6min = std::max(std::abs(jj1 - jj5), std::abs(jj4 - jj2)) / 2;
          int J6max = std::min(jj1 + jj5, jj4 + jj2) / 2;
          base[((a * d1 + b) * d1 + c) * d1 + d] = (int)tot;
          tot += (size_t)n3 * std::max(0, J6max - J6min + 1);
        }
  val.assign(tot, 0.0);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int a = 0; a < d1; ++a)
    for (int b = 0; b < d1; ++b)
      for (int c = 0; c < d1; ++c)
        for (int d = 0; d < d1; ++d) {
          int jj1 = 2 * a + 1, jj2 = 2 * b + 1, jj4 = 2 * c + 1, jj5 = 2 * d + 1;
          int J3min = std::abs(jj1 - jj2) / 2, J3max = (jj1 + jj2) / 2;
          int J6min = std::max(std::abs(jj1 - jj5), std::abs(jj4 - jj2)) / 2;
          int J6max = std::min(jj1 + jj5, jj4 + jj2) / 2;
          int n6 = J6max - J6min + 1;
          if (n6 <= 0) continue;
          size_t b0 = base[((a * d1 + b) * d1 + c) * d1 + d];
          for (int J3 = J3min; J3 <= J3max; ++J3)
            for (int J6 = J6min; J6 <= J6max; ++J6)
              val[b0 + (J3 - J3min) * n6 + (J6 - J6min)] = sixj_dd(jj1, jj2, 2 * J3, jj4, jj5, 2 * J6);
        }
}

template <class T>
T* dev_copy(TensorLayout& t, const std::vector<T>& v)
{
  void* p = nullptr;
  size_t bytes = std::max<size_t>(1, v.size()) * sizeof(T);
  if (cudaMalloc(&p, bytes) != cudaSuccess) throw std::runtime_error("cudaMalloc (tensor tables)");
  t.dev_allocs.push_back(p);
  if (!v.empty() && cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess)
    throw std::runtime_error("cudaMemcpy (tensor tables)");
  return (T*)p;
}

}  // namespace

TensorLayout::~TensorLayout()
{
  for (SplitPlan* p : {sp_lad1, sp_lad2, sp_zb1, sp_zb2})
    if (p) split_plan_destroy(p);
  for (void* p : dev_allocs) cudaFree(p);
}

// The orbit quadruples of the inverse tensor Pandya transform (k_tinv_q): a
// bra ket (i <= j) and a ket ket (k <= l) with the rank's parity and |dTz|,
// kept when some (J1, J2) gives a stored element it owns: block (chb, chk)
// with chb <= chk and, within a diagonal block, ket index >= bra index.
static void build_quadruples(const Space& s, TensorLayout& t)
{
  const int N = s.norb, nk = s.nkets, NJ = s.NJ, d1 = s.d1, lam = t.lam;
  std::vector<int> kp, kq;
  for (int p = 0; p < N; ++p)
    for (int q = p; q < N; ++q) {
      kp.push_back(p);
      kq.push_back(q);
    }
  struct Item {
    int key;
    int2 v;
  };
  std::vector<std::vector<Item>> part(nk);
  int maxj = 0;
  for (int p = 0; p < N; ++p) maxj = std::max(maxj, s.j2[p]);
#pragma omp parallel for schedule(dynamic, 16)
  for (int kb = 0; kb < nk; ++kb) {
    const int i = kp[kb], j = kq[kb];
    const int pb = (s.l[i] + s.l[j]) & 1, tb = (s.tz2[i] + s.tz2[j]) / 2;
    const int ji = s.j2[i], jj = s.j2[j];
    for (int kk = 0; kk < nk; ++kk) {
      const int k = kp[kk], l = kq[kk];
      const int pk = (s.l[k] + s.l[l]) & 1, tk = (s.tz2[k] + s.tz2[l]) / 2;
      if (((pb + pk + t.parity) & 1) || std::abs(tb - tk) != t.trank) continue;
      const int jk = s.j2[k], jl = s.j2[l];
      bool owned = false;
      for (int J1 = std::abs(ji - jj) / 2; J1 <= (ji + jj) / 2 && J1 < NJ && !owned; ++J1) {
        const int ib = s.ketJ_loc[(size_t)J1 * nk + kb];
        if (ib < 0) continue;
        const int chb = 6 * J1 + 2 * (tb + 1) + pb;
        for (int J2 = std::max(std::abs(jk - jl) / 2, std::abs(J1 - lam)); J2 <= std::min((jk + jl) / 2, J1 + lam) && J2 < NJ;
             ++J2) {
          const int ik = s.ketJ_loc[(size_t)J2 * nk + kk];
          if (ik < 0) continue;
          const int chk = 6 * J2 + 2 * (tk + 1) + pk;
          if (chb < chk || (chb == chk && ik >= ib)) {
            owned = true;
            break;
          }
        }
      }
      if (!owned) continue;
      const int key = ((((ji - 1) / 2) * d1 + (jj - 1) / 2) * d1 + (jk - 1) / 2) * d1 + (jl - 1) / 2;
      part[kb].push_back({key, make_int2(i | (j << 16), k | (l << 16))});
    }
  }
  // counting sort by class
  const int nkey = d1 * d1 * d1 * d1;
  std::vector<long long> cnt(nkey + 1, 0);
  for (const auto& v : part)
    for (const Item& it : v) ++cnt[it.key + 1];
  for (int x = 0; x < nkey; ++x) cnt[x + 1] += cnt[x];
  t.tq.assign((size_t)cnt[nkey], make_int2(0, 0));
  for (const auto& v : part)
    for (const Item& it : v) t.tq[(size_t)cnt[it.key]++] = it.v;
  t.tq_max_j3 = maxj + 1;
}

TensorLayout* tensor_layout(Space& s, int lam, int trank, int parity)
{
  const int key = (lam * 4 + trank) * 2 + parity;
  auto it = s.tensors.find(key);
  if (it != s.tensors.end()) return it->second;
  TensorLayout* t = new TensorLayout();
  t->lam = lam;
  t->trank = trank;
  t->parity = parity;
  // blocks in TwoBodyME::Allocate order
  t->lookup.assign((size_t)s.nch * s.nch, -1);
  int64_t cur = round32(32 + (int64_t)s.norb * s.norb);
  for (int cb = 0; cb < s.nch; ++cb)
    for (int ck = cb; ck < s.nch; ++ck) {
      const Chan &B = s.ch[cb], &K = s.ch[ck];
      if (std::abs(B.J - K.J) > lam || B.J + K.J < lam) continue;
      if (std::abs(B.Tz - K.Tz) != trank) continue;
      if ((B.parity + K.parity + parity) & 1) continue;
      t->lookup[(size_t)cb * s.nch + ck] = (int)t->bra.size();
      t->bra.push_back(cb);
      t->ket.push_back(ck);
      t->off.push_back(cur);
      cur = round32(cur + (int64_t)B.n() * K.n());
    }
  t->total = cur;
  for (size_t b = 0; b < t->bra.size(); ++b) {
    const int64_t nb = s.ch[t->bra[b]].n(), nk = s.ch[t->ket[b]].n();
    t->max_blk_elems = std::max<int64_t>(t->max_blk_elems, nb * nk);
    t->max_pair_elems = std::max<int64_t>(t->max_pair_elems, nb * ((nk + 1) / 2));
    t->max_tiles32 = std::max<int>(t->max_tiles32, (int)(((nb + 31) / 32) * ((nk + 31) / 32)));
  }
  for (int c = 0; c < s.nch; ++c)
    t->max_xbf = std::max<long long>(t->max_xbf, 2LL * s.cc_nph[c] * s.cc[c].n());
  // comm222_phst (src/TensorCommutators.cc:1059-1386): Zbar blocks for the
  // cross-coupled channel pairs lo <= hi allowed by the rank, and the ordered
  // pairs of the tensor Pandya transform of Y they read, (lo, hi) and (hi, lo)
  t->zb_lookup.assign((size_t)s.nch * s.nch, -1);
  t->yb_lookup.assign((size_t)s.nch * s.nch, -1);
  int64_t zc = 0, yc = 0;
  auto need_y = [&](int b, int k) {
    int64_t& slot = t->yb_lookup[(size_t)b * s.nch + k];
    if (slot >= 0) return;
    slot = yc;
    t->yb_bra.push_back(b);
    t->yb_ket.push_back(k);
    t->yb_off.push_back(yc);
    int64_t e = (int64_t)2 * s.cc_nph[b] * s.cc[k].n();
    t->yb_maxelems = (int)std::max<int64_t>(t->yb_maxelems, e);
    yc = round32(yc + e);
  };
  for (int b = 0; b < s.nch; ++b) {
    const Chan& B = s.cc[b];
    if (B.n() < 1) continue;
    for (int k = b; k < s.nch; ++k) {
      const Chan& K = s.cc[k];
      if (K.n() < 1) continue;
      if ((B.parity + K.parity + parity) & 1) continue;
      if (B.J + K.J < lam || std::abs(B.J - K.J) > lam) continue;
      if (!(B.Tz + K.Tz == trank || std::abs(B.Tz - K.Tz) == trank)) continue;
      t->zb_lookup[(size_t)b * s.nch + k] = zc;
      t->zb_bra.push_back(b);
      t->zb_ket.push_back(k);
      t->zb_off.push_back(zc);
      int64_t e = (int64_t)B.n() * 2 * K.n();
      t->zb_maxelems = (int)std::max<int64_t>(t->zb_maxelems, e);
      zc = round32(zc + e);
      need_y(b, k);
      need_y(k, b);
    }
  }
  t->zb_total = zc;
  t->yb_total = yc;
  // one-body elements: Operator::SetUpOneBodyChannels (src/Operator.cc:248-291)
  const int N = s.norb;
  t->ob_ok.assign((size_t)N * N, 0);
  for (int i = 0; i < N; ++i)
    for (int j = 0; j < N; ++j)
      t->ob_ok[(size_t)i * N + j] = ((s.l[i] + s.l[j] + parity) % 2 == 0) && triad2(s.j2[i], s.j2[j], 2 * lam) &&
                                    std::abs(s.tz2[i] - s.tz2[j]) == 2 * trank;
  // the same as lists: tob_list[tob_off[i] .. tob_off[i + 1]) = the j with ob_ok(i, j)
  t->tob_off.assign(N + 1, 0);
  t->tob_list.clear();
  for (int i = 0; i < N; ++i) {
    t->tob_off[i] = (int)t->tob_list.size();
    for (int j = 0; j < N; ++j)
      if (t->ob_ok[(size_t)i * N + j]) t->tob_list.push_back(j);
  }
  t->tob_off[N] = (int)t->tob_list.size();
  for (int i = 0; i < N; ++i) {
    t->max_tob = std::max(t->max_tob, t->tob_off[i + 1] - t->tob_off[i]);
    t->max_ob = std::max(t->max_ob, s.ob_count[i]);
  }
  // norm weights (the reference's integer arithmetic, including its mix of
  // doubled j and integer rank_J in the one-body degeneracy)
  t->nrm1_idx.clear();
  t->nrm1_w.clear();
  for (int p = 0; p < N; ++p)
    for (int q = 0; q < N; ++q) {
      if (!t->ob_ok[(size_t)q * N + p]) continue;
      const int jp = s.j2[p], jq = s.j2[q];
      const int dfac = (jp + 1) * ((std::min(jq, jp + lam) - std::max(-jq, jp - lam)) / 2 + 1);
      if (dfac == 0) continue;
      t->nrm1_idx.push_back(32 + q * N + p);  // OneBody(p, q), column-major
      t->nrm1_w.push_back((double)dfac);
    }
  t->nrm2_off.clear();
  t->nrm2_len.clear();
  t->nrm2_w.clear();
  for (size_t b = 0; b < t->bra.size(); ++b) {
    const int Jb = s.ch[t->bra[b]].J, Jk = s.ch[t->ket[b]].J;
    const long long nn = (long long)s.ch[t->bra[b]].n() * s.ch[t->ket[b]].n();
    const double deg = (double)((2 * Jk + 1) * (std::min(Jb, Jk + lam) - std::max(-Jb, Jk - lam) + 1));
    const double w = deg * deg * (t->bra[b] == t->ket[b] ? 1.0 : 2.0);
    for (long long o = 0; o < nn; o += 65536) {
      t->nrm2_off.push_back(t->off[b] + o);
      t->nrm2_len.push_back((int)std::min<long long>(65536, nn - o));
      t->nrm2_w.push_back(w);
    }
  }
  t->h_nrm_partial.assign(t->nrm2_off.size() + 1, 0.0);
  // angular tables, half-integers widened by lam (the 9j sums reach j + lam)
  t->NJ = s.NJ;
  t->d1x = s.d1 + lam;
  const int NJ = t->NJ, d1x = t->d1x;
  t->sixjA.assign((size_t)NJ * NJ * d1x * d1x * d1x, 0.0);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int I1 = 0; I1 < NJ; ++I1)
    for (int I2 = 0; I2 < NJ; ++I2) {
      if (!triad2(2 * I1, 2 * I2, 2 * lam)) continue;
      for (int a = 0; a < d1x; ++a)
        for (int b = 0; b < d1x; ++b)
          for (int c = 0; c < d1x; ++c) {
            int ja = 2 * a + 1, jb = 2 * b + 1, jc = 2 * c + 1;
            // {I1 I2 lam; ja jb jc}: triads (I1 jb jc), (ja I2 jc), (ja jb lam)
            if (!triad2(2 * I1, jb, jc) || !triad2(ja, 2 * I2, jc) || !triad2(ja, jb, 2 * lam)) continue;
            t->sixjA[((((size_t)I1 * NJ + I2) * d1x + a) * d1x + b) * d1x + c] =
                sixj_dd(2 * I1, 2 * I2, 2 * lam, ja, jb, jc);
          }
    }
  build_compact(d1x, t->sixjx_base, t->sixjx_val);
  // the 9j table (ninej_get), filled from the 6j tables above
  {
    const int d1 = s.d1, w = 2 * lam + 1;
    t->nj_d1 = d1;
    t->nj_base.assign((size_t)d1 * d1 * d1 * d1, 0);
    long long tot = 0;
    for (int a = 0; a < d1; ++a)
      for (int b = 0; b < d1; ++b)
        for (int c = 0; c < d1; ++c)
          for (int d = 0; d < d1; ++d) {
            const int ja = 2 * a + 1, jb = 2 * b + 1, jd = 2 * d + 1;
            const int nJ1 = (ja + jd - std::abs(ja - jd)) / 2 + 1, nJb = (ja + jb - std::abs(ja - jb)) / 2 + 1;
            t->nj_base[((size_t)(a * d1 + b) * d1 + c) * d1 + d] = tot;
            tot += (long long)nJ1 * w * nJb * w;
          }
    t->nj_val.assign((size_t)tot, 0.0);
    t->nj_hat.assign((size_t)tot, 0.0);
    DevTensor h = tensor_host_view(*t);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
    for (int a = 0; a < d1; ++a)
      for (int b = 0; b < d1; ++b)
        for (int c = 0; c < d1; ++c)
          for (int d = 0; d < d1; ++d) {
            const int ja = 2 * a + 1, jb = 2 * b + 1, jc = 2 * c + 1, jd = 2 * d + 1;
            const int J1min = std::abs(ja - jd) / 2, J1max = (ja + jd) / 2;
            const int Jbmin = std::abs(ja - jb) / 2, Jbmax = (ja + jb) / 2, nJb = Jbmax - Jbmin + 1;
            long long k = t->nj_base[((size_t)(a * d1 + b) * d1 + c) * d1 + d];
            for (int J1 = J1min; J1 <= J1max; ++J1)
              for (int o2 = 0; o2 < w; ++o2)
                for (int Jb = Jbmin; Jb <= Jbmax; ++Jb)
                  for (int o4 = 0; o4 < w; ++o4, ++k) {
                    const int J2 = J1 - lam + o2, Jk = Jb - lam + o4;
                    if (J2 < 0 || Jk < 0 || !triad2(jb, jc, 2 * J2) || !triad2(jd, jc, 2 * Jk)) continue;
                    const double v = ninej_tensor(h, lam, ja, jb, jc, jd, J1, J2, Jb, Jk);
                    t->nj_val[k] = v;
                    if (std::fabs(v) >= 1e-8)
                      t->nj_hat[k] = std::sqrt((double)((2 * J1 + 1) * (2 * J2 + 1) * (2 * Jb + 1) * (2 * Jk + 1))) * v;
                  }
            (void)nJb;
          }
  }
  // the scalar ladder's gather lists per channel (weights wpp - nn)
  t->lad_koff.assign(s.nch, 0);
  t->lad_woff.assign(s.nch, 0);
  t->lad_n.assign(s.nch, 0);
  for (const SymGemmJob& jb : s.ladder_jobs) {
    int c = -1;
    for (int x = 0; x < s.nch; ++x)
      if (s.ch[x].n() && s.ch[x].off == jb.a_off) c = x;
    if (c < 0) continue;
    t->lad_koff[c] = jb.kidx_off;
    t->lad_woff[c] = jb.w_off;
    t->lad_n[c] = jb.K;
    t->lad_maxelems = std::max(t->lad_maxelems, (long long)jb.m * jb.K);
  }
  build_quadruples(s, *t);
  t->hat2.assign((size_t)t->NJ * t->NJ, 0.0);
  for (int J1 = 0; J1 < t->NJ; ++J1)
    for (int J2 = 0; J2 < t->NJ; ++J2) t->hat2[(size_t)J1 * t->NJ + J2] = std::sqrt((double)((2 * J1 + 1) * (2 * J2 + 1)));
  s.tensors[key] = t;
  return t;
}

DevTensor tensor_host_view(const TensorLayout& t)
{
  DevTensor d;
  d.lam = t.lam;
  d.trank = t.trank;
  d.parity = t.parity;
  d.nblk = (int)t.bra.size();
  d.total = t.total;
  d.sixjA = t.sixjA.data();
  d.sixjx_base = t.sixjx_base.data();
  d.sixjx_val = t.sixjx_val.data();
  d.NJ = t.NJ;
  d.d1x = t.d1x;
  d.nj_base = t.nj_base.empty() ? nullptr : t.nj_base.data();
  d.nj_val = t.nj_val.empty() ? nullptr : t.nj_val.data();
  d.nj_hat = t.nj_hat.empty() ? nullptr : t.nj_hat.data();
  d.d1 = t.nj_d1;
  d.hat2 = t.hat2.data();
  d.tob_off = t.tob_off.data();
  d.tob_list = t.tob_list.data();
  d.lad_koff = t.lad_koff.data();
  d.lad_woff = t.lad_woff.data();
  d.lad_n = t.lad_n.data();
  return d;
}

void tensor_upload(TensorLayout& t)
{
  if (t.dev_ready) return;
  DevTensor& d = t.dev;
  d.lam = t.lam;
  d.trank = t.trank;
  d.parity = t.parity;
  d.nblk = (int)t.bra.size();
  d.total = t.total;
  d.bra = dev_copy(t, t.bra);
  d.ket = dev_copy(t, t.ket);
  std::vector<long long> off(t.off.begin(), t.off.end());
  d.off = dev_copy(t, off);
  d.lookup = dev_copy(t, t.lookup);
  d.ob_ok = dev_copy(t, t.ob_ok);
  d.sixjA = dev_copy(t, t.sixjA);
  d.sixjx_base = dev_copy(t, t.sixjx_base);
  d.sixjx_val = dev_copy(t, t.sixjx_val);
  d.NJ = t.NJ;
  d.d1x = t.d1x;
  d.nzb = (int)t.zb_bra.size();
  d.nyb = (int)t.yb_bra.size();
  d.zb_bra = dev_copy(t, t.zb_bra);
  d.zb_ket = dev_copy(t, t.zb_ket);
  std::vector<long long> zo(t.zb_off.begin(), t.zb_off.end()), yo(t.yb_off.begin(), t.yb_off.end());
  std::vector<long long> zl(t.zb_lookup.begin(), t.zb_lookup.end()), yl(t.yb_lookup.begin(), t.yb_lookup.end());
  d.zb_off = dev_copy(t, zo);
  d.zb_lookup = dev_copy(t, zl);
  d.yb_bra = dev_copy(t, t.yb_bra);
  d.yb_ket = dev_copy(t, t.yb_ket);
  d.yb_off = dev_copy(t, yo);
  d.yb_lookup = dev_copy(t, yl);
  d.zb_total = t.zb_total;
  d.yb_total = t.yb_total;
  d.nj_base = dev_copy(t, t.nj_base);
  d.nj_val = nullptr;  // the kernels read the hat-weighted table only
  d.nj_hat = dev_copy(t, t.nj_hat);
  d.d1 = t.nj_d1;
  d.hat2 = dev_copy(t, t.hat2);
  t.d_nrm1_idx = dev_copy(t, t.nrm1_idx);
  t.d_nrm1_w = dev_copy(t, t.nrm1_w);
  t.d_nrm2_off = dev_copy(t, t.nrm2_off);
  t.d_nrm2_len = dev_copy(t, t.nrm2_len);
  t.d_nrm2_w = dev_copy(t, t.nrm2_w);
  t.d_nrm_partial = dev_copy(t, t.h_nrm_partial);
  d.tob_off = dev_copy(t, t.tob_off);
  d.tob_list = dev_copy(t, t.tob_list);
  t.d_tq = dev_copy(t, t.tq);
  d.lad_koff = dev_copy(t, t.lad_koff);
  d.lad_woff = dev_copy(t, t.lad_woff);
  d.lad_n = dev_copy(t, t.lad_n);
  t.dev_ready = true;
}

}  // namespace imsrg
