/* Test infrastructure (oracle build only). Stand-in for GSL's gsl_math.h,
 * which the reference's Operator.cc includes without using any symbol from it
 * on the IMSRG(2) commutator path. */
#pragma once
#include <math.h>
