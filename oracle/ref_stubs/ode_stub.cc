// Test infrastructure: NOT part of the product.
//
// Stand-ins for IMSRGSolver's ODE methods, which the reference compiles only
// with Boost odeint (absent in this image; the sources are built with
// -DNO_ODE).  The Magnus solvers the harness runs never call them.
#include "IMSRGSolver.hh"

#include <cstdlib>
#include <iostream>

static void no_ode()
{
  std::cerr << "IMSRGSolver ODE methods are not built (no Boost odeint)\n";
  std::abort();
}

void IMSRGSolver::Solve_ode() { no_ode(); }
void IMSRGSolver::Solve_ode_adaptive() { no_ode(); }
void IMSRGSolver::Solve_ode_magnus() { no_ode(); }
