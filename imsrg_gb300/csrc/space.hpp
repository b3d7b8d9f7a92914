// Host-side model space of the GB300 IMSRG(2) commutator: the reference's
// ModelSpace channel bookkeeping (orbits, kets p<=q, two-body channels,
// cross-coupled channels, 6j table), the arena layout of an operator, the
// precomputed work lists of every kernel, and their device copies.
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

#include "devspace.cuh"

namespace imsrg {

struct TensorLayout;

struct Chan {
  int J = 0, parity = 0, Tz = 0;
  std::vector<int> p, q;         // kets in local order
  std::vector<int> pp, hh, ph;   // local indices by class, ascending
  int64_t off = 0;               // arena offset (2b channels only)
  int n() const { return (int)p.size(); }
};

// A dense channel product Out (+)= P + sign * phi phi^T o P^T, P = A B^T,
// evaluated on tile pairs (see kernels_gemm.cu).  Host description.
struct SymGemmJob {
  int64_t a_off = 0;   // A(i,t) = A[a_off + col(t)*lda + i]
  int64_t b_off = 0;   // B(j,t) = bscale * w(t) * B[b_off + col(t)*ldb + j]
  int64_t out_off = 0; // Out(i,j) = Out[out_off + j*ldo + i]
  int m = 0, K = 0, lda = 0, ldb = 0, ldo = 0;
  int kidx_off = -1;   // column gather list (into the space's kidx table), -1 = identity
  int w_off = -1;      // weight list (into the space's kweight table), -1 = 1
  int phase_off = -1;  // +-1 row phases (into the space's phase table), -1 = none
};

struct Space {
  // ---- orbits
  int emax = 0, norb = 0, nch = 0, nkets = 0, NJ = 0;
  std::vector<int> n, l, j2, tz2;
  std::vector<double> occ;
  std::vector<int> holes;
  std::vector<int> ob_start, ob_count, ob_list;  // one-body channel members of each orbit
  // ---- channels
  std::vector<Chan> ch, cc;
  std::vector<int> ketJ_loc;  // [J * nkets + ket] -> local index in 2b channel, -1
  std::vector<int> ccJ_loc;   // [J * nkets + ket] -> local index in CC channel, -1
  int64_t arena = 0;
  // ---- 6j table (compact, see sixj.cpp)
  int d1 = 0;
  std::vector<int> sixj_base;
  std::vector<double> sixj_val;
  std::vector<double> sixj_wval;  // (2 J6 + 1) * value, 0 where |value| < 1e-8
  std::vector<float2> sixj_wf;    // sixj_wval as (hi, lo) float pairs

  // ---- work lists
  // ladder (comm222_pp_hh): per channel, kets with nonzero weight and weights
  std::vector<int> kidx;          // flat gather lists
  std::vector<double> kweight;    // flat weights
  std::vector<int> phase_tab;     // flat +-1 row phases
  std::vector<SymGemmJob> ladder_jobs;  // one per nonempty channel (A = X, B = Y)
  std::vector<int> ladder_kidx_off, ladder_w_off;
  // Pandya: per CC channel
  std::vector<int> cc_nph;               // hh + ph kets of the CC channel
  std::vector<int> cc_ph_off;            // into cc_ph (local indices, hh then ph)
  std::vector<int> cc_ph;
  std::vector<int64_t> xb_off;           // Xbar / YbarT / YflipT: n_cc x 2nph column-major
  std::vector<int64_t> zb_off;           // Zbar: n_cc x 2 n_cc column-major
  int64_t xb_total = 0, zb_total = 0;
  std::vector<int> cc_phase_off;         // phi of each CC ket (into phase_tab)
  std::vector<SymGemmJob> zbar_jobs;     // head + tail per CC channel
  std::vector<PfOut> pf_out;             // Pandya transform of X and Y: one per panel element
  std::vector<int> pf_e;                 // its terms: arena index and signed (2J+1) 6j weight
  std::vector<double> pf_w;

  // ---- small-term work lists
  std::vector<double> ket_wpp, ket_nn;  // per 2b channel ket (flat, channel-major): Mpp / Mhh weights
  std::vector<int> hh_off, hh_list;     // per 2b channel: local indices of its hh kets
  std::vector<int> items220;            // (ch, hh local) pairs, flattened
  std::vector<int> pairs1b;             // (i, j), i <= j in one one-body channel, flattened
  std::vector<int> items221;            // (i, j, c), flattened
  std::vector<int> cols122;             // (ch, column, first item, item count), flattened
  std::vector<int> it122_loc, it122_a, it122_src;
  std::vector<double> it122_f;
  // inverse Pandya by orbit quadruple (split form, see build_invq_tasks)
  std::vector<int> cls_list, cls_off;  // orbits of each (parity, Tz) class, ascending; offsets (5)
  std::vector<unsigned char> cls_sort; // per class: positions in cls_list ordered by (2j, position)
  std::vector<int> invq_tasks;         // 4 ints per block: i | k << 16, cj | cl << 8, jf | jn << 16, lf | ln << 16
  int invq_smem = 0;                   // dynamic shared memory of the largest block (bytes)

  DevSpace dev{};     // device copies of the tables (pointers owned below)
  DevWork work{};
  std::vector<void*> dev_allocs;

  // scratch owned by the space (lazily sized)
  struct Scratch {
    void* ptr = nullptr;
    size_t bytes = 0;
  };
  Scratch s_xb, s_yb, s_yf, s_zb, s_w2, s_red, s_split_a, s_split_b, s_split_e, s_jobs;

  // tensor-operator layouts by rank, built on first use (tensor.cpp)
  std::map<int, TensorLayout*> tensors;

  ~Space();
};

// builds everything above from the orbit list; throws std::runtime_error
Space* build_space(int emax, const std::vector<int>& n, const std::vector<int>& l, const std::vector<int>& j2,
                   const std::vector<int>& tz2, const std::vector<double>& occ);
// reference orbit list of ModelSpace(emax, ref, ref)
void reference_orbits(int emax, int A, int Z, std::vector<int>& n, std::vector<int>& l, std::vector<int>& j2,
                      std::vector<int>& tz2, std::vector<double>& occ);
// copies the tables to the device (cudaMalloc); throws on failure
void upload_space(Space& s);
// blocks of the quadruple-ordered inverse Pandya transform, each within
// budget bytes of shared memory (fills cls_list, cls_off, invq_tasks, invq_smem)
void build_invq_tasks(Space& s, int budget);
// shared memory of one block of jn x ln quadruples: four 16-bit counts /
// offsets per pair, then `slot_bytes` (per staged Zbar value 8 bytes and its
// 16-bit owner, per result slot its 16-bit owner)
inline int invq_slot_bytes(int n1, int n2, int nJ) { return 10 * (n1 + n2) + 2 * nJ; }
inline int invq_block_bytes(int jn, int ln, int slot_bytes) { return ((8 * jn * ln + 15) & ~15) + slot_bytes; }

// 6j table construction (sixj.cpp)
double sixj_dd(int jj1, int jj2, int jj3, int jj4, int jj5, int jj6);  // doubled arguments
void build_sixj_table(Space& s);
double sixj_lookup(const Space& s, int jj1, int jj2, int J3, int jj4, int jj5, int J6);

}  // namespace imsrg
