// Test infrastructure: NOT part of the product.
//
// Driver that runs the reference implementation (IMSRG++ compiled from its own
// sources by oracle/ref_build.mk) on operators read from binary "arena" files
// and writes the results in the same arena layout.  It is only used in the
// build container to produce the golden fixtures under tests/golden/ and to pin
// the C oracle (oracle/imsrg_oracle.c) against the reference itself.
//
// Arena layout (doubles, shared with the product and the C oracle):
//   [0]                ZeroBody
//   [32 .. 32+N*N)     OneBody, N x N column-major (N = number of orbits)
//   then, for each two-body channel ch = 6J + 2(Tz+1) + parity in index order,
//   an n_ch x n_ch column-major block (local ket order of TwoBodyChannel),
//   every block starting on a multiple of 32 doubles.
//
// usage: ref_harness <emax> <X.bin> <Y.bin> <W.bin> <outdir>
//   X hermitian, Y anti-hermitian, W hermitian.  Writes
//     tables.txt                      orbits and channel ket lists
//     <case>_<term>.bin               term applied to a zeroed Z
//     <case>_full.bin                 Commutator::CommutatorScalarScalar
//   for the cases  xy = [X,Y] (Z hermitian), yx = [Y,X] (Z hermitian),
//   xw = [X,W] (Z anti-hermitian), and
//     bch.bin                         BCH::BCH_Transform(X, 0.25*Y/|Y|)
//     norms.txt                       Operator::Norm of the inputs
//     X_op.bin, Y_op.bin              Operator::WriteBinary of X and Y
//     pandya_{X,Y}_{normal,transpose}.bin
//                                     Commutator::DoPandyaTransformation of X
//                                     and Y: each cross-coupled channel's
//                                     matrix, column-major, in channel order
//     pandya_dims.txt                 "ch rows cols" of the normal orientation
//
// usage: ref_harness flow <emax> <H.bin> <A.bin> <B.bin> <nsteps> <outdir>
//   H hermitian (a flow Hamiltonian), A and B anti-hermitian.  Writes
//     bchp.bin                        BCH::BCH_Product(A, B)
//     bchp_big.bin                    BCH::BCH_Product(6A, 2B)
//     eta_white.bin, eta_atan.bin     Generator::Update(H, Eta), types white / atan
//     eta_white_mp.bin                white with Moller-Plesset denominators
//     flow_steps.txt                  "s E0" after each of <nsteps> Magnus-Euler
//                                     steps: IMSRGSolver(H), white generator,
//                                     ds = ds_max = 0.5, fixed step, no Omega split
//     flow_Hs.bin, flow_Omega.bin     H(s) and Omega after the last step
//     flow2_Hs.bin, flow2_Omega.bin,  the same flow with adaptive steps
//     flow2.txt                       (defaults: norm_domega 0.1, ds_max 0.5),
//                                     Omega split at |Omega| > 0.3, to s = 2:
//                                     "s nOmega E0"

#include "ModelSpace.hh"
#include "Operator.hh"
#include "Commutator.hh"
#include "BCH.hh"
#include "Generator.hh"
#include "IMSRGSolver.hh"

#include <omp.h>

#include <algorithm>
#include <cstdio>
#include <deque>
#include <cstdlib>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <string>
#include <vector>

static size_t round32(size_t x) { return (x + 31) / 32 * 32; }

struct ArenaLayout {
  size_t n_orb = 0;
  std::vector<size_t> off2;  // per channel
  std::vector<size_t> dim2;
  size_t total = 0;
};

static ArenaLayout make_layout(ModelSpace& ms) {
  ArenaLayout L;
  L.n_orb = ms.GetNumberOrbits();
  size_t cur = round32(32 + L.n_orb * L.n_orb);
  int nch = ms.GetNumberTwoBodyChannels();
  for (int ch = 0; ch < nch; ++ch) {
    size_t n = ms.GetTwoBodyChannel(ch).GetNumberKets();
    L.off2.push_back(cur);
    L.dim2.push_back(n);
    cur = round32(cur + n * n);
  }
  L.total = cur;
  return L;
}

static std::vector<double> read_file(const std::string& path, size_t expect) {
  std::vector<double> v(expect, 0.0);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) { std::cerr << "cannot open " << path << "\n"; std::exit(2); }
  size_t got = std::fread(v.data(), sizeof(double), expect, f);
  std::fclose(f);
  if (got != expect) { std::cerr << path << ": expected " << expect << " doubles, got " << got << "\n"; std::exit(2); }
  return v;
}

static void write_file(const std::string& path, const std::vector<double>& v) {
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::cerr << "cannot write " << path << "\n"; std::exit(2); }
  std::fwrite(v.data(), sizeof(double), v.size(), f);
  std::fclose(f);
}

static void load(Operator& op, const std::vector<double>& a, const ArenaLayout& L) {
  op.ZeroBody = a[0];
  for (size_t c = 0; c < L.n_orb; ++c)
    for (size_t r = 0; r < L.n_orb; ++r) op.OneBody(r, c) = a[32 + c * L.n_orb + r];
  for (size_t ch = 0; ch < L.off2.size(); ++ch) {
    size_t n = L.dim2[ch];
    if (n == 0) continue;
    arma::mat& M = op.TwoBody.GetMatrix(ch, ch);
    for (size_t c = 0; c < n; ++c)
      for (size_t r = 0; r < n; ++r) M(r, c) = a[L.off2[ch] + c * n + r];
  }
}

static std::vector<double> store(const Operator& op, const ArenaLayout& L) {
  std::vector<double> a(L.total, 0.0);
  a[0] = op.ZeroBody;
  for (size_t c = 0; c < L.n_orb; ++c)
    for (size_t r = 0; r < L.n_orb; ++r) a[32 + c * L.n_orb + r] = op.OneBody(r, c);
  for (size_t ch = 0; ch < L.off2.size(); ++ch) {
    size_t n = L.dim2[ch];
    if (n == 0) continue;
    const arma::mat& M = op.TwoBody.GetMatrix(ch, ch);
    for (size_t c = 0; c < n; ++c)
      for (size_t r = 0; r < n; ++r) a[L.off2[ch] + c * n + r] = M(r, c);
  }
  return a;
}

static void dump_tables(ModelSpace& ms, const std::string& path) {
  std::ofstream out(path);
  int norb = ms.GetNumberOrbits();
  out << "orbits " << norb << "\n";
  for (int i = 0; i < norb; ++i) {
    Orbit& o = ms.GetOrbit(i);
    out << i << " " << o.n << " " << o.l << " " << o.j2 << " " << o.tz2 << " " << std::setprecision(17) << o.occ << "\n";
  }
  int nch = ms.GetNumberTwoBodyChannels();
  out << "channels " << nch << "\n";
  for (int ch = 0; ch < nch; ++ch) {
    TwoBodyChannel& tbc = ms.GetTwoBodyChannel(ch);
    int n = tbc.GetNumberKets();
    out << ch << " " << tbc.J << " " << tbc.parity << " " << tbc.Tz << " " << n;
    for (int i = 0; i < n; ++i) out << " " << tbc.GetKet(i).p << " " << tbc.GetKet(i).q;
    out << "\n";
    out << "pp " << tbc.GetKetIndex_pp().n_elem;
    for (auto x : tbc.GetKetIndex_pp()) out << " " << x;
    out << "\nhh " << tbc.GetKetIndex_hh().n_elem;
    for (auto x : tbc.GetKetIndex_hh()) out << " " << x;
    out << "\nph " << tbc.GetKetIndex_ph().n_elem;
    for (auto x : tbc.GetKetIndex_ph()) out << " " << x;
    out << "\n";
  }
  out << "cc_channels " << nch << "\n";
  for (int ch = 0; ch < nch; ++ch) {
    TwoBodyChannel_CC& tbc = ms.GetTwoBodyChannel_CC(ch);
    int n = tbc.GetNumberKets();
    out << ch << " " << tbc.J << " " << tbc.parity << " " << tbc.Tz << " " << n;
    for (int i = 0; i < n; ++i) out << " " << tbc.GetKet(i).p << " " << tbc.GetKet(i).q;
    out << "\n";
    out << "hh " << tbc.GetKetIndex_hh().n_elem;
    for (auto x : tbc.GetKetIndex_hh()) out << " " << x;
    out << "\nph " << tbc.GetKetIndex_ph().n_elem;
    for (auto x : tbc.GetKetIndex_ph()) out << " " << x;
    out << "\n";
  }
}

typedef void (*term_fn)(const Operator&, const Operator&, Operator&);

static size_t tensor_total(const Operator& op, size_t n_orb) {
  size_t cur = round32(32 + n_orb * n_orb);
  for (auto& it : op.TwoBody.MatEl) cur = round32(cur + it.second.n_elem);
  return cur;
}

static void load_tensor(Operator& op, const std::vector<double>& a, size_t n_orb) {
  op.ZeroBody = a[0];
  for (size_t c = 0; c < n_orb; ++c)
    for (size_t r = 0; r < n_orb; ++r) op.OneBody(r, c) = a[32 + c * n_orb + r];
  size_t cur = round32(32 + n_orb * n_orb);
  for (auto& it : op.TwoBody.MatEl) {
    arma::mat& M = it.second;
    for (size_t e = 0; e < M.n_elem; ++e) M.memptr()[e] = a[cur + e];
    cur = round32(cur + M.n_elem);
  }
}

static std::vector<double> store_tensor(const Operator& op, size_t n_orb) {
  std::vector<double> a(tensor_total(op, n_orb), 0.0);
  a[0] = op.ZeroBody;
  for (size_t c = 0; c < n_orb; ++c)
    for (size_t r = 0; r < n_orb; ++r) a[32 + c * n_orb + r] = op.OneBody(r, c);
  size_t cur = round32(32 + n_orb * n_orb);
  for (auto& it : op.TwoBody.MatEl) {
    const arma::mat& M = it.second;
    for (size_t e = 0; e < M.n_elem; ++e) a[cur + e] = M.memptr()[e];
    cur = round32(cur + M.n_elem);
  }
  return a;
}

static int tensor_main(int argc, char** argv) {
  if (argc != 10 && argc != 11) {
    std::cerr << "usage: ref_harness tensor <emax> <lam> <trank> <parity> <herm> <X.bin> <T.bin> <outdir> [nucleus]\n";
    return 1;
  }
  int emax = std::atoi(argv[2]), lam = std::atoi(argv[3]), trank = std::atoi(argv[4]), parity = std::atoi(argv[5]);
  int herm = std::atoi(argv[6]);
  std::string outdir = argv[9];
  const std::string nucleus = argc == 11 ? argv[10] : "O16";
  ModelSpace ms(emax, nucleus, nucleus);
  ArenaLayout L = make_layout(ms);
  size_t N = L.n_orb;
  Operator X(ms, 0, 0, 0, 2);
  X.SetHermitian();
  load(X, read_file(argv[7], L.total), L);
  Operator T(ms, lam, trank, parity, 2);
  if (herm > 0) T.SetHermitian(); else T.SetAntiHermitian();
  load_tensor(T, read_file(argv[8], tensor_total(T, N)), N);
  {
    std::ofstream bf(outdir + "/tensor_blocks.txt");
    for (auto& it : T.TwoBody.MatEl)
      bf << it.first[0] << " " << it.first[1] << " " << it.second.n_rows << " " << it.second.n_cols << "\n";
  }
  struct Term { const char* name; term_fn fn; };
  const Term terms[] = {
      {"comm111st", Commutator::comm111st},
      {"comm121st", Commutator::comm121st},
      {"comm122st", Commutator::comm122st},
      {"comm222_pp_hh_221st", Commutator::comm222_pp_hh_221st},
      {"comm222_phst", Commutator::comm222_phst},
  };
  for (const Term& t : terms) {
    Operator Z(ms, lam, trank, parity, 2);
    if (herm > 0) Z.SetAntiHermitian(); else Z.SetHermitian();
    t.fn(X, T, Z);
    write_file(outdir + "/st_" + t.name + ".bin", store_tensor(Z, N));
  }
  Operator Zf = Commutator::CommutatorScalarTensor(X, T);
  write_file(outdir + "/st_full.bin", store_tensor(Zf, N));
  // BCH_Transform of the tensor by Omega = 0.2 X / |X|, and the norms
  {
    Operator Omega = X * (0.2 / X.Norm());
    write_file(outdir + "/st_omega.bin", store(Omega, L));
    Operator B = BCH::BCH_Transform(T, Omega);
    write_file(outdir + "/st_bch.bin", store_tensor(B, N));
    std::ofstream nf(outdir + "/st_norms.txt");
    nf << std::setprecision(17) << T.Norm() << " " << Zf.Norm() << " " << B.Norm() << " " << T.OneBodyNorm() << " "
       << T.TwoBodyNorm() << "\n";
  }
  {
    // Operator::WriteBinary of the tensor
    std::ofstream ot(outdir + "/st_T_op.bin", std::ios::binary);
    T.WriteBinary(ot);
  }
  return 0;
}

static int flow_main(int argc, char** argv) {
  if (argc != 8) {
    std::cerr << "usage: ref_harness flow <emax> <H.bin> <A.bin> <B.bin> <nsteps> <outdir>\n";
    return 1;
  }
  int emax = std::atoi(argv[2]);
  int nsteps = std::atoi(argv[6]);
  std::string outdir = argv[7];
  ModelSpace ms(emax, "O16", "O16");
  ArenaLayout L = make_layout(ms);
  Operator H(ms, 0, 0, 0, 2), A(ms, 0, 0, 0, 2), B(ms, 0, 0, 0, 2);
  H.SetHermitian();
  A.SetAntiHermitian();
  B.SetAntiHermitian();
  load(H, read_file(argv[3], L.total), L);
  load(A, read_file(argv[4], L.total), L);
  load(B, read_file(argv[5], L.total), L);

  write_file(outdir + "/bchp.bin", store(BCH::BCH_Product(A, B), L));
  {
    Operator A6 = A * 6.0;
    Operator B2 = B * 2.0;
    write_file(outdir + "/bchp_big.bin", store(BCH::BCH_Product(A6, B2), L));
  }

  struct GenCase { const char* file; const char* type; const char* part; };
  const GenCase gens[] = {{"eta_white", "white", "Epstein_Nesbet"},
                          {"eta_atan", "atan", "Epstein_Nesbet"},
                          {"eta_white_mp", "white", "Moller_Plesset"},
                          {"eta_qt", "qtransfer-atan", "Epstein_Nesbet"},
                          {"eta_qt2", "qtransfer-atan_2", "Epstein_Nesbet"}};
  for (const GenCase& g : gens) {
    Generator gen;
    gen.SetType(g.type);
    gen.SetDenominatorPartitioning(g.part);
    Operator Eta(H);
    Eta.Erase();
    Eta.SetAntiHermitian();
    gen.Update(H, Eta);
    write_file(outdir + "/" + g.file + ".bin", store(Eta, L));
  }

  {
    IMSRGSolver solver(H);
    solver.SetGenerator("white");
    solver.SetDs(0.5);
    solver.SetDsmax(0.5);
    solver.SetMagnusAdaptive(false);
    solver.SetOmegaNormMax(1e9);
    solver.SetEtaCriterion(1e-20);
    std::ofstream f(outdir + "/flow_steps.txt");
    f << std::setprecision(17);
    for (int k = 1; k <= nsteps; ++k) {
      solver.SetSmax(0.5 * k);
      solver.Solve();
      f << solver.GetS() << " " << solver.GetH_s().ZeroBody << "\n";
    }
    write_file(outdir + "/flow_Hs.bin", store(solver.GetH_s(), L));
    write_file(outdir + "/flow_Omega.bin", store(solver.GetOmega(solver.GetOmegaSize() - 1), L));
  }
  {
    IMSRGSolver solver(H);
    solver.SetGenerator("white");
    solver.SetOmegaNormMax(0.3);
    solver.SetEtaCriterion(1e-20);
    solver.SetSmax(2.0);
    solver.Solve();
    std::ofstream f(outdir + "/flow2.txt");
    f << std::setprecision(17) << solver.GetS() << " " << solver.GetOmegaSize() << " " << solver.GetH_s().ZeroBody
      << "\n";
    write_file(outdir + "/flow2_Hs.bin", store(solver.GetH_s(), L));
    write_file(outdir + "/flow2_Omega.bin", store(solver.GetOmega(solver.GetOmegaSize() - 1), L));
  }
  // the other solver methods: Magnus modified Euler and back-off, with Omega
  // splits, and the fixed-step RK4 flow of H itself
  struct MethodCase { const char* name; const char* method; };
  const MethodCase methods[] = {
      {"flow_me", "magnus_modified_euler"}, {"flow_bo", "magnus_backoff"}, {"flow_rk4", "flow_RK4"}};
  // flow_RK4 also flows an added observable, the hermitian [A, H]
  Operator obs = Commutator::Commutator(A, H);
  for (const MethodCase& mc : methods) {
    const bool rk4 = std::string(mc.method) == "flow_RK4";
    IMSRGSolver solver(H);
    solver.SetGenerator("white");
    solver.SetMethod(mc.method);
    solver.SetOmegaNormMax(0.3);
    solver.SetEtaCriterion(1e-20);
    solver.SetSmax(2.0);
    if (rk4) solver.AddOperator(obs);
    solver.Solve();
    std::ofstream f(outdir + "/" + mc.name + ".txt");
    f << std::setprecision(17) << solver.GetS() << " " << solver.GetOmegaSize() << " " << solver.GetH_s().ZeroBody
      << "\n";
    write_file(outdir + "/" + mc.name + "_Hs.bin", store(solver.GetH_s(), L));
    if (rk4) {
      write_file(outdir + "/flow_rk4_obs_in.bin", store(obs, L));
      write_file(outdir + "/flow_rk4_obs.bin", store(solver.GetOperator(1), L));
    }
  }
  return 0;
}

// usage: ref_harness time <emax> <X.bin> <Y.bin> <reps>
//   Commutator::CommutatorScalarScalar(X, Y) once untimed (6j tables, first
//   touches), then reps times; prints "seconds_per_commutator <t> threads <n>".
static int time_main(int argc, char** argv) {
  if (argc != 6) {
    std::cerr << "usage: ref_harness time <emax> <X.bin> <Y.bin> <reps>\n";
    return 1;
  }
  int emax = std::atoi(argv[2]);
  int reps = std::atoi(argv[5]);
  ModelSpace ms(emax, "O16", "O16");
  ArenaLayout L = make_layout(ms);
  Operator X(ms, 0, 0, 0, 2), Y(ms, 0, 0, 0, 2);
  X.SetHermitian();
  Y.SetAntiHermitian();
  load(X, read_file(argv[3], L.total), L);
  load(Y, read_file(argv[4], L.total), L);
  Operator Z = Commutator::CommutatorScalarScalar(X, Y);
  double t0 = omp_get_wtime();
  for (int r = 0; r < reps; ++r) Z = Commutator::CommutatorScalarScalar(X, Y);
  double t = (omp_get_wtime() - t0) / std::max(1, reps);
  std::cout << "seconds_per_commutator " << std::setprecision(6) << t << " threads " << omp_get_max_threads()
            << "\n";
  return 0;
}

int main(int argc, char** argv) {
  if (argc > 1 && std::string(argv[1]) == "time") return time_main(argc, argv);
  if (argc > 1 && std::string(argv[1]) == "flow") return flow_main(argc, argv);
  if (argc > 1 && std::string(argv[1]) == "tensor") return tensor_main(argc, argv);
  if (argc != 6) {
    std::cerr << "usage: ref_harness <emax> <X.bin> <Y.bin> <W.bin> <outdir>\n";
    return 1;
  }
  int emax = std::atoi(argv[1]);
  std::string outdir = argv[5];
  ModelSpace ms(emax, "O16", "O16");
  ArenaLayout L = make_layout(ms);
  dump_tables(ms, outdir + "/tables.txt");

  Operator X(ms, 0, 0, 0, 2), Y(ms, 0, 0, 0, 2), W(ms, 0, 0, 0, 2);
  X.SetHermitian();
  Y.SetAntiHermitian();
  W.SetHermitian();
  load(X, read_file(argv[2], L.total), L);
  load(Y, read_file(argv[3], L.total), L);
  load(W, read_file(argv[4], L.total), L);

  {
    std::ofstream nf(outdir + "/norms.txt");
    nf << std::setprecision(17) << X.Norm() << " " << Y.Norm() << " " << W.Norm() << "\n";
  }
  {
    // Operator::WriteBinary of X and Y (the E2max field is written from an
    // uninitialised member there, src/Operator.cc:65-75; readers skip it)
    std::ofstream ox(outdir + "/X_op.bin", std::ios::binary);
    X.WriteBinary(ox);
    std::ofstream oy(outdir + "/Y_op.bin", std::ios::binary);
    Y.WriteBinary(oy);
  }

  struct Term { const char* name; term_fn fn; };
  const Term terms[] = {
      {"comm110ss", Commutator::comm110ss},
      {"comm220ss", Commutator::comm220ss},
      {"comm111ss", Commutator::comm111ss},
      {"comm121ss", Commutator::comm121ss},
      {"comm122ss", Commutator::comm122ss},
      {"comm222_pp_hh_221ss", Commutator::comm222_pp_hh_221ss},
      {"comm222_pp_hhss", Commutator::comm222_pp_hhss},
      {"comm221ss", Commutator::comm221ss},
      {"comm222_phss", Commutator::comm222_phss},
  };
  struct Case { const char* name; const Operator* a; const Operator* b; bool z_herm; };
  const Case cases[] = {{"xy", &X, &Y, true}, {"yx", &Y, &X, true}, {"xw", &X, &W, false}};

  for (const Case& cs : cases) {
    for (const Term& t : terms) {
      Operator Z(ms, 0, 0, 0, 2);
      if (cs.z_herm) Z.SetHermitian(); else Z.SetAntiHermitian();
      t.fn(*cs.a, *cs.b, Z);
      write_file(outdir + "/" + cs.name + "_" + t.name + ".bin", store(Z, L));
    }
    Operator Zf = Commutator::CommutatorScalarScalar(*cs.a, *cs.b);
    write_file(outdir + "/" + cs.name + "_full.bin", store(Zf, L));
  }

  Operator Omega = Y * (0.25 / Y.Norm());
  Operator Hs = BCH::BCH_Transform(X, Omega);
  write_file(outdir + "/bch.bin", store(Hs, L));

  // single-operator Pandya transform of X and Y, both orientations: every
  // cross-coupled channel's matrix, column-major, concatenated in channel order
  {
    std::ofstream dims(outdir + "/pandya_dims.txt");
    struct PCase { const char* name; const Operator* op; const char* orient; };
    const PCase pcs[] = {{"X_normal", &X, "normal"}, {"X_transpose", &X, "transpose"},
                         {"Y_normal", &Y, "normal"}, {"Y_transpose", &Y, "transpose"}};
    for (const PCase& pc : pcs) {
      std::deque<arma::mat> mats(ms.GetNumberTwoBodyChannels());
      Commutator::DoPandyaTransformation(*pc.op, mats, pc.orient);
      std::vector<double> flat;
      for (size_t ch = 0; ch < mats.size(); ++ch) {
        const arma::mat& M = mats[ch];
        if (pc.op == &X && std::string(pc.orient) == "normal") dims << ch << " " << M.n_rows << " " << M.n_cols << "\n";
        flat.insert(flat.end(), M.memptr(), M.memptr() + M.n_elem);
      }
      write_file(outdir + "/pandya_" + pc.name + ".bin", flat);
    }
  }
  return 0;
}
