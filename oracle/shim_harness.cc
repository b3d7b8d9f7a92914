// Test infrastructure: NOT part of the product.
//
// Driver of the drop-in link (oracle/ref_build.mk, target shim): IMSRG++
// compiled from its own sources, with imsrg_gb300/shim/imsrg_gpu_shim.cc
// linked in place of Commutator::comm*ss, Commutator::CommutatorScalarScalar
// and BCH::Standard_BCH_Transform.
//
// usage: shim_harness layout <emax>
//   builds ModelSpace(emax, "O16", "O16") and checks, through the shim, that
//   the GPU space's channels and kets are the reference's (host only).
// usage: shim_harness dispatch <emax>
//   calls the reference's own entry points (Commutator::comm*ss,
//   Commutator::Commutator, BCH::BCH_Transform) and reports which
//   implementation answered: on a machine without a GPU the shim's calls
//   fail with an "imsrg_gb300:" error, which the reference's would not.
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <stdexcept>
#include <string>

#include "BCH.hh"
#include "Commutator.hh"
#include "ModelSpace.hh"
#include "Operator.hh"

extern "C" int imsrg_gpu_shim_layout_check(ModelSpace* ms);

typedef void (*term_fn)(const Operator&, const Operator&, Operator&);

static std::string answered(const std::string& what, void (*call)())
{
  try {
    call();
  } catch (std::exception& e) {
    if (std::strncmp(e.what(), "imsrg_gb300:", 12) == 0) return what + " imsrg_gb300";
    return what + " error " + e.what();
  }
  return what + " reference";
}

static ModelSpace* g_ms = nullptr;
static Operator* g_X = nullptr;
static Operator* g_Y = nullptr;
static term_fn g_term = nullptr;

int main(int argc, char** argv)
{
  if (argc != 3) {
    std::cerr << "usage: shim_harness layout|dispatch <emax>\n";
    return 1;
  }
  const std::string mode = argv[1];
  ModelSpace ms(std::atoi(argv[2]), "O16", "O16");
  g_ms = &ms;
  if (mode == "layout") {
    int bad = imsrg_gpu_shim_layout_check(&ms);
    std::cout << (bad ? "layout mismatches " + std::to_string(bad) : std::string("layout ok")) << "\n";
    return bad ? 1 : 0;
  }
  if (mode != "dispatch") return 1;
  Operator X(ms, 0, 0, 0, 2), Y(ms, 0, 0, 0, 2);
  X.SetHermitian();
  Y.SetAntiHermitian();
  g_X = &X;
  g_Y = &Y;
  const struct {
    const char* name;
    term_fn fn;
  } terms[] = {{"comm110ss", Commutator::comm110ss},     {"comm220ss", Commutator::comm220ss},
               {"comm111ss", Commutator::comm111ss},     {"comm121ss", Commutator::comm121ss},
               {"comm122ss", Commutator::comm122ss},     {"comm221ss", Commutator::comm221ss},
               {"comm222_pp_hhss", Commutator::comm222_pp_hhss},
               {"comm222_pp_hh_221ss", Commutator::comm222_pp_hh_221ss},
               {"comm222_phss", Commutator::comm222_phss}};
  for (auto& t : terms) {
    g_term = t.fn;
    std::cout << answered(t.name, [] {
      Operator Z(*g_ms, 0, 0, 0, 2);
      Z.SetHermitian();
      g_term(*g_X, *g_Y, Z);
    }) << "\n";
  }
  std::cout << answered("Commutator::Commutator", [] { Commutator::Commutator(*g_X, *g_Y); }) << "\n";
  std::cout << answered("BCH::BCH_Transform", [] { BCH::BCH_Transform(*g_X, *g_Y); }) << "\n";
  return 0;
}
