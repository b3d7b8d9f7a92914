/* Test infrastructure: NOT part of the product.
 *
 * Wigner 3j / 6j / 9j symbols with the signature of GSL's coupling functions
 * (gsl_sf_coupling_3j/6j/9j, GSL is not installed in this image).  They stand
 * in for GSL when the reference is compiled into the oracle (the reference
 * calls them from src/AngMom.cc:84,96,102) and they give the C oracle
 * (oracle/imsrg_oracle.c) its recoupling coefficients.
 *
 * Algorithms (published closed forms, restated here):
 *   3j: Racah's single-sum formula (Edmonds, "Angular Momentum in Quantum
 *       Mechanics", eq. 3.7.3).
 *   6j: Racah's single-sum formula (Edmonds eq. 6.3.7).
 *   9j: sum over x of three 6j symbols (Edmonds eq. 6.4.3).
 * Arguments are twice the angular momenta.  The sums run in long double on
 * factorials tabulated in long double.
 */
#include <math.h>
#include <stdlib.h>

#define CPL_FACT_MAX 170

static long double cpl_fact_tab[CPL_FACT_MAX + 1];
static int cpl_fact_ready = 0;

static long double cpl_fact(int n)
{
  if (!cpl_fact_ready) {
    long double f = 1.0L;
    cpl_fact_tab[0] = 1.0L;
    for (int i = 1; i <= CPL_FACT_MAX; ++i) {
      f *= (long double)i;
      cpl_fact_tab[i] = f;
    }
    cpl_fact_ready = 1;
  }
  if (n < 0 || n > CPL_FACT_MAX) return 0.0L;
  return cpl_fact_tab[n];
}

/* triad (a,b,c) in doubled units: |a-b| <= c <= a+b and a+b+c even */
static int cpl_triad(int a, int b, int c)
{
  if (a < 0 || b < 0 || c < 0) return 0;
  if ((a + b + c) & 1) return 0;
  if (c > a + b) return 0;
  if (c < abs(a - b)) return 0;
  return 1;
}

/* Delta(abc)^2 with doubled arguments */
static long double cpl_delta2(int a, int b, int c)
{
  return cpl_fact((a + b - c) / 2) * cpl_fact((a - b + c) / 2) * cpl_fact((-a + b + c) / 2) /
         cpl_fact((a + b + c) / 2 + 1);
}

double gsl_sf_coupling_6j(int ja, int jb, int jc, int jd, int je, int jf)
{
  if (!cpl_triad(ja, jb, jc) || !cpl_triad(ja, je, jf) || !cpl_triad(jd, jb, jf) || !cpl_triad(jd, je, jc))
    return 0.0;
  int a1 = (ja + jb + jc) / 2, a2 = (ja + je + jf) / 2, a3 = (jd + jb + jf) / 2, a4 = (jd + je + jc) / 2;
  int b1 = (ja + jb + jd + je) / 2, b2 = (ja + jc + jd + jf) / 2, b3 = (jb + jc + je + jf) / 2;
  int tmin = a1;
  if (a2 > tmin) tmin = a2;
  if (a3 > tmin) tmin = a3;
  if (a4 > tmin) tmin = a4;
  int tmax = b1;
  if (b2 < tmax) tmax = b2;
  if (b3 < tmax) tmax = b3;
  long double sum = 0.0L;
  for (int t = tmin; t <= tmax; ++t) {
    long double den = cpl_fact(t - a1) * cpl_fact(t - a2) * cpl_fact(t - a3) * cpl_fact(t - a4) *
                      cpl_fact(b1 - t) * cpl_fact(b2 - t) * cpl_fact(b3 - t);
    long double term = cpl_fact(t + 1) / den;
    sum += (t & 1) ? -term : term;
  }
  long double pre = sqrtl(cpl_delta2(ja, jb, jc) * cpl_delta2(ja, je, jf) * cpl_delta2(jd, jb, jf) *
                          cpl_delta2(jd, je, jc));
  return (double)(pre * sum);
}

double gsl_sf_coupling_3j(int ja, int jb, int jc, int ma, int mb, int mc)
{
  if (!cpl_triad(ja, jb, jc)) return 0.0;
  if (ma + mb + mc != 0) return 0.0;
  if (abs(ma) > ja || abs(mb) > jb || abs(mc) > jc) return 0.0;
  if (((ja + ma) & 1) || ((jb + mb) & 1) || ((jc + mc) & 1)) return 0.0;
  /* doubled -> integer combinations */
  int k1 = (ja + jb - jc) / 2; /* j1+j2-j3 */
  int k2 = (ja - ma) / 2;      /* j1-m1 */
  int k3 = (jb + mb) / 2;      /* j2+m2 */
  int k4 = (jc - jb + ma) / 2; /* j3-j2+m1 */
  int k5 = (jc - ja - mb) / 2; /* j3-j1-m2 */
  int kmin = 0;
  if (-k4 > kmin) kmin = -k4;
  if (-k5 > kmin) kmin = -k5;
  int kmax = k1;
  if (k2 < kmax) kmax = k2;
  if (k3 < kmax) kmax = k3;
  long double sum = 0.0L;
  for (int k = kmin; k <= kmax; ++k) {
    long double den = cpl_fact(k) * cpl_fact(k1 - k) * cpl_fact(k2 - k) * cpl_fact(k3 - k) *
                      cpl_fact(k4 + k) * cpl_fact(k5 + k);
    sum += (k & 1) ? -1.0L / den : 1.0L / den;
  }
  long double pre = sqrtl(cpl_delta2(ja, jb, jc) * cpl_fact((ja + ma) / 2) * cpl_fact((ja - ma) / 2) *
                          cpl_fact((jb + mb) / 2) * cpl_fact((jb - mb) / 2) * cpl_fact((jc + mc) / 2) *
                          cpl_fact((jc - mc) / 2));
  int ph = (ja - jb - mc) / 2; /* j1-j2-m3 */
  long double v = pre * sum;
  return (double)((ph & 1) ? -v : v);
}

double gsl_sf_coupling_9j(int ja, int jb, int jc, int jd, int je, int jf, int jg, int jh, int ji)
{
  if (!cpl_triad(ja, jb, jc) || !cpl_triad(jd, je, jf) || !cpl_triad(jg, jh, ji) ||
      !cpl_triad(ja, jd, jg) || !cpl_triad(jb, je, jh) || !cpl_triad(jc, jf, ji))
    return 0.0;
  int xmin = abs(ja - ji);
  if (abs(jh - jd) > xmin) xmin = abs(jh - jd);
  if (abs(jb - jf) > xmin) xmin = abs(jb - jf);
  int xmax = ja + ji;
  if (jh + jd < xmax) xmax = jh + jd;
  if (jb + jf < xmax) xmax = jb + jf;
  long double sum = 0.0L;
  for (int x = xmin; x <= xmax; x += 2) {
    long double s = (long double)gsl_sf_coupling_6j(ja, jb, jc, jf, ji, x) *
                    (long double)gsl_sf_coupling_6j(jd, je, jf, jb, x, jh) *
                    (long double)gsl_sf_coupling_6j(jg, jh, ji, x, ja, jd);
    sum += (x & 1 ? -1.0L : 1.0L) * (x + 1) * s; /* (-1)^{2x} with x doubled */
  }
  return (double)sum;
}
