// 6j symbols for the recoupling kernels.
//
// Values: Racah's single-sum formula (Edmonds, "Angular Momentum in Quantum
// Mechanics", eq. 6.3.7) evaluated in double-double arithmetic (pairs of
// IEEE doubles, Dekker / Knuth error-free transformations), so the
// alternating sum keeps ~100 bits before the final rounding to double.
// This file must be compiled with -ffp-contract=off: the error-free
// transformations rely on every product and sum being rounded separately
// (the one fused operation used is the explicit std::fma in two_prod).
//
// Storage: the reference keeps a dense table SixJCache_112112 indexed by
// (jj1, jj2, J3, jj4, jj5, J6) (src/AngMomCache.hh:15-47, 54 MiB at emax 10).
// Here only the triad-allowed window is stored: for each (jj1, jj2, jj4, jj5),
// J3 in [|j1-j2|, j1+j2] times J6 in [max(|j1-j5|,|j4-j2|), min(j1+j5, j4+j2)],
// about 10x smaller, so the table stays in L2 next to the operator tiles.
#include <cmath>
#include <cstdlib>
#include <vector>

#include "space.hpp"

namespace imsrg {
namespace {

struct dd {
  double hi, lo;
};

inline dd two_sum(double a, double b)
{
  double s = a + b;
  double bb = s - a;
  double e = (a - (s - bb)) + (b - bb);
  return {s, e};
}

inline dd quick_two_sum(double a, double b)
{
  double s = a + b;
  double e = b - (s - a);
  return {s, e};
}

inline dd two_prod(double a, double b)
{
  double p = a * b;
  double e = std::fma(a, b, -p);
  return {p, e};
}

inline dd dd_add(dd a, dd b)
{
  dd s = two_sum(a.hi, b.hi);
  dd t = two_sum(a.lo, b.lo);
  s.lo += t.hi;
  s = quick_two_sum(s.hi, s.lo);
  s.lo += t.lo;
  return quick_two_sum(s.hi, s.lo);
}

inline dd dd_mul(dd a, dd b)
{
  dd p = two_prod(a.hi, b.hi);
  p.lo += a.hi * b.lo + a.lo * b.hi;
  return quick_two_sum(p.hi, p.lo);
}

inline dd dd_div(dd a, dd b)
{
  double q1 = a.hi / b.hi;
  dd r = dd_add(a, dd_mul(b, dd{-q1, 0.0}));
  double q2 = r.hi / b.hi;
  r = dd_add(r, dd_mul(b, dd{-q2, 0.0}));
  double q3 = r.hi / b.hi;
  dd q = quick_two_sum(q1, q2);
  return dd_add(q, dd{q3, 0.0});
}

inline dd dd_sqrt(dd a)
{
  if (a.hi <= 0.0) return {0.0, 0.0};
  double x = std::sqrt(a.hi);
  dd xx = two_prod(x, x);
  dd r = dd_add(a, dd{-xx.hi, -xx.lo});
  return quick_two_sum(x, r.hi / (2.0 * x));
}

const std::vector<dd>& factorials()
{
  static std::vector<dd> f = [] {
    std::vector<dd> v(171);
    v[0] = {1.0, 0.0};
    for (int i = 1; i <= 170; ++i) v[i] = dd_mul(v[i - 1], dd{(double)i, 0.0});
    return v;
  }();
  return f;
}

inline dd fact(int n) { return factorials()[n]; }

inline bool triad(int a, int b, int c)
{
  if ((a + b + c) & 1) return false;
  return c <= a + b && c >= std::abs(a - b);
}

inline dd delta2(int a, int b, int c)
{
  dd num = dd_mul(dd_mul(fact((a + b - c) / 2), fact((a - b + c) / 2)), fact((-a + b + c) / 2));
  return dd_div(num, fact((a + b + c) / 2 + 1));
}

}  // namespace

double sixj_dd(int ja, int jb, int jc, int jd, int je, int jf)
{
  if (!triad(ja, jb, jc) || !triad(ja, je, jf) || !triad(jd, jb, jf) || !triad(jd, je, jc)) return 0.0;
  int a1 = (ja + jb + jc) / 2, a2 = (ja + je + jf) / 2, a3 = (jd + jb + jf) / 2, a4 = (jd + je + jc) / 2;
  int b1 = (ja + jb + jd + je) / 2, b2 = (ja + jc + jd + jf) / 2, b3 = (jb + jc + je + jf) / 2;
  int tmin = std::max(std::max(a1, a2), std::max(a3, a4));
  int tmax = std::min(b1, std::min(b2, b3));
  dd sum{0.0, 0.0};
  for (int t = tmin; t <= tmax; ++t) {
    dd den = dd_mul(dd_mul(dd_mul(fact(t - a1), fact(t - a2)), dd_mul(fact(t - a3), fact(t - a4))),
                    dd_mul(dd_mul(fact(b1 - t), fact(b2 - t)), fact(b3 - t)));
    dd term = dd_div(fact(t + 1), den);
    if (t & 1) term = {-term.hi, -term.lo};
    sum = dd_add(sum, term);
  }
  dd pre2 = dd_mul(dd_mul(delta2(ja, jb, jc), delta2(ja, je, jf)), dd_mul(delta2(jd, jb, jf), delta2(jd, je, jc)));
  dd v = dd_mul(dd_sqrt(pre2), sum);
  return v.hi + v.lo;
}

void build_sixj_table(Space& s)
{
  int jjmax = 2 * s.emax + 1;
  for (int j : s.j2) jjmax = std::max(jjmax, j);
  int d1 = (jjmax - 1) / 2 + 1;
  s.d1 = d1;
  s.sixj_base.assign((size_t)d1 * d1 * d1 * d1, 0);
  // sizes first
  size_t tot = 0;
  for (int a = 0; a < d1; ++a)
    for (int b = 0; b < d1; ++b)
      for (int c = 0; c < d1; ++c)
        for (int d = 0; d < d1; ++d) {
          int jj1 = 2 * a + 1, jj2 = 2 * b + 1, jj4 = 2 * c + 1, jj5 = 2 * d + 1;
          int n3 = ((jj1 + jj2) - std::abs(jj1 - jj2)) / 2 + 1;
          int J6min = std::max(std::abs(jj1 - jj5), std::abs(jj4 - jj2)) / 2;
          int J6max = std::min(jj1 + jj5, jj4 + jj2) / 2;
          int n6 = std::max(0, J6max - J6min + 1);
          s.sixj_base[((a * d1 + b) * d1 + c) * d1 + d] = (int)tot;
          tot += (size_t)n3 * n6;
        }
  s.sixj_val.assign(tot, 0.0);
#pragma omp parallel for schedule(dynamic, 1) collapse(2)
  for (int a = 0; a < d1; ++a)
    for (int b = 0; b < d1; ++b)
      for (int c = 0; c < d1; ++c)
        for (int d = 0; d < d1; ++d) {
          int jj1 = 2 * a + 1, jj2 = 2 * b + 1, jj4 = 2 * c + 1, jj5 = 2 * d + 1;
          int J3min = std::abs(jj1 - jj2) / 2, J3max = (jj1 + jj2) / 2;
          int J6min = std::max(std::abs(jj1 - jj5), std::abs(jj4 - jj2)) / 2;
          int J6max = std::min(jj1 + jj5, jj4 + jj2) / 2;
          int base = s.sixj_base[((a * d1 + b) * d1 + c) * d1 + d];
          int n6 = J6max - J6min + 1;
          if (n6 <= 0) continue;
          for (int J3 = J3min; J3 <= J3max; ++J3)
            for (int J6 = J6min; J6 <= J6max; ++J6)
              s.sixj_val[base + (J3 - J3min) * n6 + (J6 - J6min)] = sixj_dd(jj1, jj2, 2 * J3, jj4, jj5, 2 * J6);
        }
  s.sixj_wval.assign(tot, 0.0);
  for (int a = 0; a < d1; ++a)
    for (int b = 0; b < d1; ++b)
      for (int c = 0; c < d1; ++c)
        for (int d = 0; d < d1; ++d) {
          int jj1 = 2 * a + 1, jj2 = 2 * b + 1, jj4 = 2 * c + 1, jj5 = 2 * d + 1;
          int J3min = std::abs(jj1 - jj2) / 2, J3max = (jj1 + jj2) / 2;
          int J6min = std::max(std::abs(jj1 - jj5), std::abs(jj4 - jj2)) / 2;
          int J6max = std::min(jj1 + jj5, jj4 + jj2) / 2;
          int base = s.sixj_base[((a * d1 + b) * d1 + c) * d1 + d];
          int n6 = J6max - J6min + 1;
          if (n6 <= 0) continue;
          for (int J3 = J3min; J3 <= J3max; ++J3)
            for (int J6 = J6min; J6 <= J6max; ++J6) {
              size_t k = base + (J3 - J3min) * n6 + (J6 - J6min);
              double v = s.sixj_val[k];
              s.sixj_wval[k] = std::fabs(v) < 1e-8 ? 0.0 : (2 * J6 + 1) * v;
            }
        }
  // (hi, lo) float pairs of the weights for the double-float kernels
  s.sixj_wf.resize(tot);
  for (size_t k = 0; k < tot; ++k) {
    float hi = (float)s.sixj_wval[k];
    s.sixj_wf[k] = float2{hi, (float)(s.sixj_wval[k] - (double)hi)};
  }
}

double sixj_lookup(const Space& s, int jj1, int jj2, int J3, int jj4, int jj5, int J6)
{
  if (jj1 < 1 || jj2 < 1 || jj4 < 1 || jj5 < 1) return 0.0;
  int dmax = 2 * s.d1 - 1;
  if (jj1 > dmax || jj2 > dmax || jj4 > dmax || jj5 > dmax) return 0.0;
  if (!(jj1 & 1) || !(jj2 & 1) || !(jj4 & 1) || !(jj5 & 1)) return 0.0;
  int slot = sixj_slot(s.d1, s.sixj_base.data(), jj1, jj2, J3, jj4, jj5, J6);
  return slot < 0 ? 0.0 : s.sixj_val[slot];
}

}  // namespace imsrg
