/* Test infrastructure (oracle build only). Declares the three GSL coupling
 * functions the reference calls from src/AngMom.cc:84,96,102 (GSL itself is
 * not installed). Arguments are twice the angular momenta, as in GSL.
 * Implemented in coupling_stub.c from the Racah formulas. */
#pragma once
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_coupling_3j(int two_ja, int two_jb, int two_jc, int two_ma, int two_mb, int two_mc);
double gsl_sf_coupling_6j(int two_ja, int two_jb, int two_jc, int two_jd, int two_je, int two_jf);
double gsl_sf_coupling_9j(int two_ja, int two_jb, int two_jc, int two_jd, int two_je, int two_jf,
                          int two_jg, int two_jh, int two_ji);
#ifdef __cplusplus
}
#endif
