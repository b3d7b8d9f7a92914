/*
 * imsrg_gb300 -- C ABI of the GB300 (sm_103a) IMSRG(2) scalar commutator.
 *
 * Drop-in boundary for IMSRG++'s angular-momentum-coupled IMSRG(2)
 * commutator [X,Y] and BCH transform.  Plain C types only: pointers, sizes,
 * int status codes, and an opaque cudaStream_t passed as void* (NULL = the
 * legacy default stream).  No entry point exits the process; every one
 * returns IMSRG_OK or an error code, with a message in imsrg_last_error().
 *
 * Data model.  A model space (imsrg_space) holds the orbit list and the
 * channel bookkeeping of the reference's ModelSpace, and the device tables
 * the kernels read.  An operator (imsrg_op) is one device-resident FP64
 * "arena" (the reference's Operator: ZeroBody, OneBody, TwoBody):
 *     [0]                 ZeroBody
 *     [32, 32+N*N)        OneBody, N x N column-major (N orbits)
 *     offset(ch) ...      one n_ch x n_ch column-major block per two-body
 *                         channel ch = 6J + 2(Tz+1) + parity, kets in the
 *                         reference's local order; every block starts on a
 *                         multiple of 32 doubles.
 * Column-major n x n blocks are exactly arma::mat, so packing a reference
 * Operator is one memcpy per block.
 *
 * Term entry points accumulate into Z, as the reference's
 * Commutator::comm*ss(X, Y, Z) do; Z's hermiticity flag selects the
 * symmetrisation.  X and Y must be hermitian or anti-hermitian.
 *
 * All calls that take the same imsrg_space share its scratch workspace and
 * must be ordered on one stream (or otherwise serialised by the caller).
 */
#ifndef IMSRG_GB300_H
#define IMSRG_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define IMSRG_OK 0
#define IMSRG_ERR_ARG 1         /* bad argument (null, size, index) */
#define IMSRG_ERR_CUDA 2        /* a CUDA runtime call failed */
#define IMSRG_ERR_UNSUPPORTED 3 /* operator symmetry the GPU path does not handle */
#define IMSRG_ERR_NOMEM 4       /* device allocation failed */
#define IMSRG_ERR_KERNEL 5      /* a kernel reported an error through its status word */
#define IMSRG_ERR_DIVERGED 6    /* the IMSRG flow blew up (|eta| > 1e12 or |E0| > 1e9) */
#define IMSRG_ERR_IO 7          /* a file could not be opened, read or written */

/* precision of the dense contractions (ladder and Pandya channel GEMMs) */
#define IMSRG_PREC_FP64 0  /* plain FP64 (CUDA-core DFMA) */
#define IMSRG_PREC_SPLIT 1 /* Ozaki-style sliced BF16 tensor-core products (tcgen05), FP64 recombination */

/* generator functions (src/Generator.cc:12-15) and energy-denominator
 * partitionings (src/Generator.cc:23-28) */
#define IMSRG_GEN_WHITE 0          /* Hod / denominator (the default) */
#define IMSRG_GEN_ATAN 1           /* atan(2 Hod / denominator) / 2 */
#define IMSRG_GEN_WEGNER 2         /* Hod * denominator */
#define IMSRG_GEN_IMAGINARY_TIME 3 /* Hod * sign(denominator) */
/* qtransfer-atan_n (qtransfer-atan is n = 1): the atan generator times
 * (|denominator| M_N / (hbar c)^2)^(n/2), 1 <= n <= 16 */
#define IMSRG_GEN_QTRANSFER_ATAN(n) (100 + (n))
#define IMSRG_DENOM_EPSTEIN_NESBET 0
#define IMSRG_DENOM_MOLLER_PLESSET 1
/* denominator_delta_index that adds denominator_delta to every denominator */
#define IMSRG_DELTA_ALL (-12345)

typedef struct imsrg_space imsrg_space;
typedef struct imsrg_op imsrg_op;
typedef struct imsrg_solver imsrg_solver;
typedef struct imsrg_batch imsrg_batch;

/* Last error message of the calling thread ("" if none). */
const char* imsrg_last_error(void);

/* ----------------------------------------------------------------- spaces */

/* Model space from an explicit orbit list (orbit i = (n[i], l[i], j2[i], tz2[i])
 * with occupation occ[i], in the reference's orbit order).  Builds kets p<=q,
 * the two-body channels, the cross-coupled channels and the 6j table.
 * Replaces ModelSpace::Init / SetupKets (src/ModelSpace.cc:353-417,1120-1200),
 * TwoBodyChannel(_CC)::Initialize (src/TwoBodyChannel.cc:19-67) and the
 * SixJCache_112112 fill (src/AngMomCache.cc:58-104).  emax bounds the 6j table
 * (orbit j2 <= 2*emax+1). */
int imsrg_space_create(int emax, int norb, const int* n, const int* l, const int* j2, const int* tz2,
                       const double* occ, imsrg_space** out);

/* Harmonic-oscillator space with every orbit 2n+l <= emax, both isospins,
 * occupations of the reference nucleus (A, Z) filled as
 * ModelSpace(emax, "<A,Z>", "<A,Z>") does (src/ModelSpace.cc:202-220,610-645). */
int imsrg_space_create_reference(int emax, int A, int Z, imsrg_space** out);

void imsrg_space_destroy(imsrg_space* s);

/* Sizes: orbits, two-body channels, arena length in doubles. */
int imsrg_space_sizes(const imsrg_space* s, int* norb, int* nch, long long* arena_len);

/* Orbit i: ModelSpace::GetOrbit (src/ModelSpace.hh:41-57). */
int imsrg_space_orbit(const imsrg_space* s, int i, int* n, int* l, int* j2, int* tz2, double* occ);

/* Two-body channel ch: TwoBodyChannel (J, parity, Tz, GetNumberKets), plus its
 * arena offset in doubles.  src/ModelSpace.cc:1046-1053, src/TwoBodyChannel.cc:19-67. */
int imsrg_space_channel(const imsrg_space* s, int ch, int* J, int* parity, int* Tz, int* nkets, long long* offset);

/* Kets of channel ch in local order: TwoBodyChannel::GetKet(i).p / .q
 * (src/TwoBodyChannel.cc:79-80).  p and q hold nkets entries each. */
int imsrg_space_channel_kets(const imsrg_space* s, int ch, int* p, int* q);

/* Cross-coupled channel ch: TwoBodyChannel_CC (src/TwoBodyChannel.cc:160-188);
 * p, q may be NULL, else hold nkets entries. */
int imsrg_space_cc_channel(const imsrg_space* s, int ch, int* J, int* parity, int* Tz, int* nkets, int* p, int* q);

/* 6j symbol {jj1/2 jj2/2 j3; jj4/2 jj5/2 j6} from the space's table
 * (ModelSpace::GetCachedSixJ, src/ModelSpace.hh:502-505; arguments doubled for
 * the half-integers, as there). */
int imsrg_space_sixj(const imsrg_space* s, int jj1, int jj2, int j3, int jj4, int jj5, int j6, double* out);

/* Layout of a Pandya-transform buffer (imsrg_pandya_transform): total
 * length in doubles, and for cross-coupled channel ch_cc (ch_cc < 0: total
 * only) its matrix's rows = 2 nph (hh then ph kets of the channel, in both
 * orders) and cols = the channel's kets, starting at offset. */
int imsrg_space_pandya_layout(const imsrg_space* s, int ch_cc, int* rows, int* cols, long long* offset,
                              long long* total);

/* -------------------------------------------------------------- operators */

/* Device-resident scalar operator (J=0, parity +, Tz=0, particle rank 2),
 * zero-filled.  hermiticity: +1 hermitian, -1 anti-hermitian.
 * Replaces Operator(ms, 0, 0, 0, 2) + SetHermitian/SetAntiHermitian
 * (src/Operator.cc:57-80, src/Operator.hh:45-225). */
int imsrg_op_create(imsrg_space* s, int hermiticity, imsrg_op** out);
void imsrg_op_destroy(imsrg_op* op);
int imsrg_op_hermiticity(const imsrg_op* op, int* h);
int imsrg_op_set_hermiticity(imsrg_op* op, int h);

/* Reduced tensor operator of rank lam (J), trank (|delta Tz|, 0 or 1) and
 * parity (0, 1), zero-filled: Operator(ms, lam, trank, parity, 2)
 * (src/Operator.cc:65-84) with reduced matrix elements.  Its arena: ZeroBody
 * at [0], OneBody N x N column-major at [32] (<i||T||j>, nonzero where
 * Operator::SetUpOneBodyChannels allows), then every TwoBodyME block
 * (ch_bra <= ch_ket allowed by the rank, in TwoBodyME::Allocate order,
 * src/TwoBodyME.cc:77-95) n_bra x n_ket column-major, each on a multiple of 32
 * doubles (imsrg_space_tensor_layout).  Blocks with ch_bra > ch_ket are the
 * conjugates: <a|T|b> = h (-1)^(J_bra - J_ket) <b|T|a>.  Upload, download,
 * zero, copy, scale and axpy take tensor operators like scalar ones (copy and
 * axpy between equal ranks); norm, random fill, files, BCH and the flow take
 * scalar operators only. */
int imsrg_op_create_tensor(imsrg_space* s, int lam, int trank, int parity, int hermiticity, imsrg_op** out);
/* rank of an operator (0, 0, 0 for scalars) and its arena length in doubles */
int imsrg_op_rank(const imsrg_op* op, int* lam, int* trank, int* parity, long long* arena_len);
/* Tensor arena layout of rank (lam, trank, parity): number of two-body blocks
 * and total length; for block >= 0 also its channels and offset. */
int imsrg_space_tensor_layout(imsrg_space* s, int lam, int trank, int parity, int block, int* ch_bra, int* ch_ket,
                              long long* offset, int* nblocks, long long* total);
/* 9j symbol {ja/2 jd/2 J1; jb/2 jc/2 J2; Jbra Jket lam} (half-integers
 * doubled) as the scalar-tensor kernels read it: the layout's 9j table, filled
 * by a sum over three 6j symbols from the space's tables (AngMom::NineJ's
 * counterpart, src/AngMom.cc:96-104); 0 outside the orbits' j range. */
int imsrg_space_ninej(imsrg_space* s, int lam, int ja, int jd, int J1, int jb, int jc, int J2, int Jbra, int Jket,
                      double* out);

/* Self-test of the failure path of the split products' bounded waits: one
 * kernel waits on an mbarrier that nothing arrives on, through the products'
 * own wait loop bounded at `limit` iterations (1 .. the production bound,
 * returned in *production_limit), sets the space's status word and returns;
 * the call reports it as IMSRG_ERR_KERNEL and clears the word, and *cycles
 * holds the SM clock cycles the wait took.  The context stays usable.  No
 * counterpart in the reference. */
int imsrg_space_wait_selftest(imsrg_space* s, unsigned limit, long long* cycles, unsigned* production_limit,
                              void* stream);

/* Host <-> device copies of the whole arena (arena_len doubles). */
int imsrg_op_upload(imsrg_op* op, const double* host, void* stream);
int imsrg_op_download(const imsrg_op* op, double* host, void* stream);
/* Device address of the arena (for callers that manage their own copies). */
int imsrg_op_device_arena(const imsrg_op* op, double** dptr);

/* Operator::Erase (src/Operator.cc), copy-assignment, operator*= and
 * operator+=(a * x) (src/Operator.cc:132-210). */
int imsrg_op_zero(imsrg_op* op, void* stream);
int imsrg_op_copy(imsrg_op* dst, const imsrg_op* src, void* stream);
int imsrg_op_scale(imsrg_op* op, double a, void* stream);
int imsrg_op_axpy(imsrg_op* y, double a, const imsrg_op* x, void* stream);

/* Operator::WriteBinary / ReadBinary (src/Operator.cc:341-388,
 * src/TwoBodyME.cc:812-836): the operator in the reference's binary layout
 * (Operator header, ZeroBody, OneBody, TwoBodyME header, every channel block
 * column-major in channel order), so files interchange with IMSRG++.  The
 * E2max field is written as 2 emax (the reference writes an uninitialised
 * value there) and ignored on reading.  Tensor operators write their rank in
 * both headers and their blocks in TwoBodyME::MatEl order.  Reading checks the
 * header against the operator (rank (J, T, parity), two-body, channel count,
 * exact length) and sets the operator's hermiticity from the file.  Both stream the arena through pinned
 * staging buffers on stream and return when the file is complete. */
int imsrg_op_write_binary(const imsrg_op* op, const char* path, void* stream);
int imsrg_op_read_binary(imsrg_op* op, const char* path, void* stream);

/* Operator::Norm (src/Operator.cc:1610-1651, src/TwoBodyME.cc:703-723) of a
 * scalar or tensor operator (a tensor's one-body elements weighted by the
 * reference's degeneracy factor, its blocks by (2Jket+1)(..)^2 and twice when
 * the bra and ket channels differ); synchronises the stream. */
int imsrg_op_norm(const imsrg_op* op, double* out, void* stream);

/* Seeded random operator: uniform[-1,1] on symmetry-allowed entries,
 * (anti)symmetrised by the operator's hermiticity, unit Frobenius norm per
 * two-body channel block and for the one-body matrix; ZeroBody uniform
 * (hermitian) or 0.  Generated on the host, then uploaded.  The test fixture
 * generator of the benchmark; UnitTest::RandomOp (src/UnitTest.cc:25-205) is
 * the reference's counterpart. */
int imsrg_op_fill_random(imsrg_op* op, unsigned long long seed, void* stream);

/* ------------------------------------------------------------------ terms */
/* Each accumulates its part of [X,Y] into Z, like the reference function
 * named in its comment.  Z must be hermitian or anti-hermitian. */

/* Commutator::comm110ss, src/Commutator.cc:564-581 */
int imsrg_comm110ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* Commutator::comm220ss, src/Commutator.cc:601-631 */
int imsrg_comm220ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* Commutator::comm111ss, src/Commutator.cc:644-649 */
int imsrg_comm111ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* Commutator::comm121ss, src/Commutator.cc:670-728 */
int imsrg_comm121ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* Commutator::comm122ss, src/Commutator.cc:837-932 */
int imsrg_comm122ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* comm122ss (plain FP64 form) that allocates no device memory, for callers
 * that cannot call cudaMalloc where they evaluate the term: code under a fixed
 * device-memory budget, a caching allocator that owns all device memory, or a
 * region where allocating is not allowed.  X, Y, Z are caller-owned device
 * arenas of the space's layout (Z accumulates); hZ is Z's hermiticity.  The
 * W2 intermediate lives in a static device array of 2^21 doubles (16 MiB)
 * that every GPU loading the library holds until exit, so spaces with a
 * longer arena are rejected (IMSRG_ERR_ARG).  Set-up is done when the space's
 * device tables are built (its first imsrg_op_create, with that device
 * current): it looks up the array's device address and loads the kernels,
 * and under lazy module loading that step may commit the array's 16 MiB.
 * Calls must be made with that same device current (IMSRG_ERR_ARG otherwise).
 * All calls share the array: calls that overlap on the GPU race.  No
 * counterpart in the reference. */
int imsrg_comm122ss_noalloc(const imsrg_space* s, const double* X, const double* Y, double* Z, int hZ, void* stream);
/* Commutator::comm221ss, src/Commutator.cc:760-819 */
int imsrg_comm221ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* Commutator::comm222_pp_hhss, src/Commutator.cc:1062-1076 */
int imsrg_comm222_pp_hhss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);
/* Commutator::comm222_pp_hh_221ss, src/Commutator.cc:1215-1301 */
int imsrg_comm222_pp_hh_221ss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);
/* Commutator::comm222_phss, src/Commutator.cc:1681-1823 */
int imsrg_comm222_phss(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);

/* ------------------------------------------------------- scalar-tensor */
/* Commutator::CommutatorScalarTensor (src/Commutator.cc:432-500) in IMSRG(2):
 * Z = [X, Y] for X scalar and Y a reduced tensor; Z, a tensor operator of Y's
 * rank, is overwritten and its hermiticity set from X and Y.  precision
 * selects the form of the ladder and Pandya-space (Z bar) products, as for the
 * scalar commutator: IMSRG_PREC_FP64, or IMSRG_PREC_SPLIT (tensor cores; the call
 * then synchronises the stream and checks the kernels' status word, as the
 * scalar entry points do); every other sum is FP64. */
int imsrg_commutator_scalar_tensor(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);
/* its terms, each accumulating into Z (src/TensorCommutators.cc) */
/* comm111st, src/TensorCommutators.cc:25-30 */
int imsrg_comm111st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* comm121st, src/TensorCommutators.cc:46-150 */
int imsrg_comm121st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* comm122st, src/TensorCommutators.cc:158-312 */
int imsrg_comm122st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, void* stream);
/* comm222_pp_hh_221st, src/TensorCommutators.cc:314-495 */
int imsrg_comm222_pp_hh_221st(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);
/* comm222_phst, src/TensorCommutators.cc:1059-1386, with the tensor Pandya
 * transforms of :637-752 and :754-920 */
int imsrg_comm222_phst(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);

/* Commutator::DoPandyaTransformation(Z, TwoBody_CC_ph, orientation),
 * src/Commutator.cc:1319-1390,1487-1497: the Pandya (particle-hole) transform
 * of one operator in every cross-coupled channel,
 *   Zbar(ab, cd) = - sum_J (2J+1) {ja jb Jcc; jc jd J} Z^J_{ad,cb}
 * (|6j| < 1e-8 skipped).  transpose = 0: the "normal" orientation, rows x
 * cols column-major (imsrg_space_pandya_layout); transpose = 1: "transpose",
 * cols x rows column-major, times herm (n_a - n_b).  out is a device buffer of
 * the layout's total length (zeroed first).  Not on the commutator's own path
 * (comm222_phss transforms X and Y together, in its own layout). */
int imsrg_pandya_transform(const imsrg_op* Z, int transpose, double* out, void* stream);

/* Layout of a Z bar buffer (imsrg_add_inverse_pandya): total length in
 * doubles, and for cross-coupled channel ch_cc (ch_cc < 0: total only) its
 * matrix's rows = the channel's kets and cols = twice that (the "head" half
 * [0, rows) and the "tail" half [rows, 2 rows) of comm222_phss's Z bar,
 * src/Commutator.cc:1789-1805), column-major from offset. */
int imsrg_space_zbar_layout(const imsrg_space* s, int ch_cc, int* rows, int* cols, long long* offset,
                            long long* total);

/* Commutator::AddInversePandyaTransformation (src/Commutator.cc:1501-1616):
 * Z += the inverse Pandya transform of zbar, a device buffer of the
 * imsrg_space_zbar_layout layout; Z's hermiticity selects the symmetrisation.
 * precision selects the kernel that comm222_phss uses in that form
 * (imsrg_space_set_tuning "inverse.split" / "inverse.fp64").  zbar must have
 * the symmetry of comm222_phss's Z bar, which every kernel relies on: head
 * Zbar(r, c) = hZ Zbar(c, r), tail Zbar(r, n + c) = phi_r phi_c Zbar(c, n + r)
 * with phi of a ket (p, q) = (-1)^((j_p + j_q) / 2); the descriptor kernels
 * read only each block's upper triangle. */
int imsrg_add_inverse_pandya(const double* zbar, imsrg_op* Z, int precision, void* stream);

/* Commutator::CommutatorScalarScalar, src/Commutator.cc:280-428 (IMSRG(2)
 * terms): Z is overwritten with [X,Y] and its hermiticity set from X and Y;
 * the terms switched on by imsrg_set_term run in the reference's order. */
int imsrg_commutator_scalar_scalar(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, int precision, void* stream);

/* Commutator::TurnOnTerm / TurnOffTerm (src/Commutator.cc:77-78) for the
 * IMSRG(2) names "comm110ss", "comm220ss", "comm111ss", "comm121ss",
 * "comm122ss", "comm221ss", "comm222_pp_hhss", "comm222_phss", and the
 * scalar-tensor names "comm111st", "comm121st", "comm122st",
 * "comm222_pp_hhst", "comm221st", "comm222_phst" (comm222_pp_hh_221st runs
 * when both comm222_pp_hhst and comm221st are on, as in the reference).
 * Process-wide. */
int imsrg_set_term(const char* name, int on);
int imsrg_get_term(const char* name, int* on);

/* Batched commutators: n independent Z[i] = [X[i], Y[i]] (each as
 * imsrg_commutator_scalar_scalar), of any mix of model spaces and sizes,
 * recorded once into a CUDA graph and replayed by imsrg_batch_launch.  Pairs
 * that share a model space run one after the other (they share its scratch);
 * pairs of different spaces run concurrently, one graph branch per space.
 * With every term on and one model space per pair, every kernel of the
 * commutator (both dense products included) runs as one grouped launch for
 * all pairs whose spaces have the same orbits and whose operators the same
 * hermiticities, in either precision (the FP64 form needs the descriptor
 * inverse Pandya kernel, "inverse.fp64" = 1, as tuned).
 * Creating a batch evaluates every pair once (allocating all scratch) and
 * captures the graph; the operators, their spaces and the term switches are
 * fixed from then on, and every operator must outlive the batch.  No Z may
 * appear twice.  No reference counterpart (the reference evaluates
 * commutators one at a time). */
int imsrg_batch_create(int n, const imsrg_op* const* X, const imsrg_op* const* Y, imsrg_op* const* Z, int precision,
                       imsrg_batch** out);
void imsrg_batch_destroy(imsrg_batch* batch);
/* Enqueue one replay of the whole batch on stream (asynchronous). */
int imsrg_batch_launch(imsrg_batch* batch, void* stream);
/* Synchronise stream and, in split precision, check the kernels' status words. */
int imsrg_batch_sync(imsrg_batch* batch, void* stream);
/* Pairs, graph branches (distinct model spaces), groups of pairs whose
 * products run as one launch (0 when products run per pair) and kernel nodes
 * per replay. */
int imsrg_batch_info(const imsrg_batch* batch, int* n_pairs, int* n_branches, int* n_product_groups,
                     long long* kernel_nodes);

/* Tuning of a space's kernels: tile shapes, pipeline depth and tile-to-CTA
 * schedules of the split products, and the inverse Pandya kernel and its
 * block sizes.  Parameters (value 0 = the built-in default where allowed):
 *   "ladder.tile", "zbar.tile"          64 (64-column tiles; consecutive
 *                                       tiles share part of tensor memory) or
 *                                       32 (32-column tiles, sharing none)
 *   "ladder.stages", "zbar.stages"      pipeline stages, 2..6 (0: most that fit)
 *   "ladder.schedule", "zbar.schedule"  0: tiles dealt round-robin to the
 *                                       persistent CTAs in size order, 1:
 *                                       longest-first greedy lists per CTA
 *   "inverse.split"                     split form: 0 orbit-quadruple blocks,
 *                                       1 descriptors with double-float sums,
 *                                       2 descriptors with FP64 sums
 *   "inverse.fp64"                      FP64 form: 0 channel tiles, 1
 *                                       descriptors (FP64 sums)
 *   "inverse.quad_budget"               shared-memory bytes per quadruple block
 *   "inverse.desc_stage", "inverse.desc_results"
 *                                       staged values / results per descriptor block
 *   "inverse.desc_weights"              1: descriptor blocks stage their 6j
 *                                       weight rows in shared memory
 *   "inverse.desc_ilp"                  results each thread of the descriptor
 *                                       kernel keeps in flight: 1, 2 or 4
 *   "ladder.digits", "zbar.digits"      digits per operand of the split
 *                                       products, 5..7 (0: as many as 36 bits
 *                                       need at the digit width that keeps the
 *                                       leading FP32 sums exact); the width
 *                                       times the count is the precision
 *   "comm122.fused"                     split-form comm122ss: 1 forms W2 tile
 *                                       pairs in shared memory and updates Z
 *                                       directly (no W2 array)
 * When the space's device tables are built (its first operator), the line of
 * the tuning file whose "arena=" and "norb=" match the space is applied: the
 * file is $IMSRG_GB300_TUNING ("off" for none), else tuning/gb300.txt in the
 * directory above the library's (written by python -m imsrg_gb300.autotune).
 * Setting a parameter drops the plans it shapes (rebuilt on next use); no
 * call on the space may be running.  The reference has no counterpart (its
 * schedule is OpenMP's dynamic one over size-sorted channels,
 * src/ModelSpace.cc:1183-1198, src/Commutator.cc:1113-1115). */
int imsrg_space_set_tuning(imsrg_space* s, const char* name, int value);
int imsrg_space_get_tuning(const imsrg_space* s, const char* name, int* value);
/* "source=<file:line | set | default> name=value ..."; with buf == NULL
 * returns the size needed */
int imsrg_space_describe_tuning(const imsrg_space* s, char* buf, int buflen);

/* Status reads of the split-precision kernels.  By default every commutator
 * and term entry point that runs a split-precision product ends by reading
 * the space's kernel status word (a 4-byte device-to-host copy and a stream
 * synchronisation), so a bounded wait that gave up is reported by the call
 * that ran it.  With defer = 1 those entry points return without the read and
 * without synchronising, so a caller can queue many commutators on a stream;
 * imsrg_space_check_status then synchronises the stream and returns
 * IMSRG_ERR_KERNEL if any kernel reported an error since the last read
 * (clearing the word).  BCH, BCH_Product, the batch and the solver read the
 * word with the norms they synchronise for anyway, whatever the setting.  No
 * counterpart in the reference (it has no device status). */
int imsrg_space_defer_status(imsrg_space* s, int defer);
int imsrg_space_check_status(imsrg_space* s, void* stream);

/* Default precision used by the reference-signature shim (process-wide). */
int imsrg_set_default_precision(int precision);
int imsrg_get_default_precision(int* precision);

/* BCH::Standard_BCH_Transform (src/BCH.cc:87-201): OpOut = e^Omega OpIn e^-Omega
 * by nested commutators, stopping as the reference does (threshold:
 * BCH::bch_transform_threshold, default 1e-9, src/BCH.cc:8-69; at most 40
 * nested commutators).  Omega is scalar; OpIn and OpOut are scalar or tensor
 * operators of one rank (a tensor's nested commutators are
 * CommutatorScalarTensor).  n_nested (may be NULL) receives the number of
 * nested commutators evaluated.  Synchronises the stream once per nested
 * commutator for the convergence test. */
int imsrg_bch_transform(const imsrg_op* OpIn, const imsrg_op* Omega, imsrg_op* OpOut, double threshold,
                        int precision, int* n_nested, void* stream);

/* BCH::BCH_Product (src/BCH.cc:267-350): Z with e^Z = e^X e^Y,
 * Z = X + Y + 1/2 [X,Y] + 1/12 ([X,[X,Y]] + [Y,[Y,X]]) + ..., nested [Y, .]
 * commutators with Bernoulli coefficients while their norm exceeds threshold
 * (BCH::bch_product_threshold, default 1e-4; at most 8 nested terms); the
 * [X,[X,Y]] term only when |[Y,X]| |X| > threshold.  Z may alias X or Y and
 * takes X's hermiticity (Operator Z = X + Y).  n_commutators (may be NULL)
 * receives the number of commutators evaluated.  Synchronises the stream once
 * per commutator.  The factorized three-body correction (off by default in the
 * reference) is not on the GPU path. */
int imsrg_bch_product(const imsrg_op* X, const imsrg_op* Y, imsrg_op* Z, double threshold, int precision,
                      int* n_commutators, void* stream);

/* -------------------------------------------------------------- generator */
/* Generator::Update(H, Eta) (src/Generator.cc:32-76) for the single-reference
 * generators (ConstructGenerator_SingleRef, :236-297): Eta is overwritten with
 * an anti-hermitian operator that is zero except <i|Eta|a> for core orbit a
 * and non-core i, and <ij|Eta|kl> for non-core i, j and core k, l; each is
 * type's function of H's element and its energy denominator
 * (Get1bDenominator / Get2bDenominator, :110-188: Epstein-Nesbet adds the
 * monopoles of H; |denominator| < cutoff is replaced by cutoff; delta is added
 * to the denominators selected by delta_index: IMSRG_DELTA_ALL for all, an
 * orbit index for the one-body ones touching that orbit, -1 for none).  The
 * core is the set of occupied orbits (the reference's core for a
 * single-reference space, src/ModelSpace.cc:278-280).  Reference defaults:
 * cutoff 1e-6, delta 0, delta_index -1.  MP_isospin partitioning and the
 * shell-model / Hartree-Fock / three-body generators are not on the GPU path. */
int imsrg_generator_update(const imsrg_op* H, imsrg_op* Eta, int type, int partitioning, double cutoff,
                           double delta, int delta_index, void* stream);

/* ----------------------------------------------------------------- solver */
/* IMSRGSolver (src/IMSRGSolver.hh:35-210) with the Magnus-Euler method
 * (Solve_magnus_euler, src/IMSRGSolver.cc:236-321), every operator in device
 * memory.  The solver refers to H0, which must outlive it unchanged; it owns
 * H(s), Eta and the Omegas (no scratch files: IMSRGSolver::NewOmega keeps
 * earlier Omegas in device memory).  Defaults are IMSRGSolver(H)'s:
 * ds 0.1, ds_max 0.5, smax 2, domega 0.1, omega_norm_max 2, eta_criterion
 * 1e-6, adaptive steps, White generator, Epstein-Nesbet denominators. */
int imsrg_solver_create(const imsrg_op* H0, imsrg_solver** out);
void imsrg_solver_destroy(imsrg_solver* solver);
/* Settings by name, the IMSRGSolver / Generator / BCH setters:
 * "ds" (SetDs), "ds_max" (SetDsmax), "smax" (SetSmax), "domega" (SetdOmega),
 * "omega_norm_max", "eta_criterion" (stored as float, as SetEtaCriterion
 * does), "magnus_adaptive", "hunter_gatherer" (0/1), "denominator_cutoff",
 * "denominator_delta", "denominator_delta_index", "bch_transform_threshold",
 * "bch_product_threshold", "max_omega_written", "method" (SetMethod: 0
 * magnus_euler, 1 magnus_modified_euler, 2 magnus_backoff, 3 flow_RK4; the
 * boost::odeint methods are not on the GPU path), "ds_backoff_factor" (0.5) and
 * "ds_max_growth_factor" (1.2) of magnus_backoff.  imsrg_solver_get also reads "s" (flow parameter),
 * "n_omega" (Omegas kept) and "istep" (steps of the last solve, + 1). */
int imsrg_solver_set(imsrg_solver* solver, const char* name, double value);
int imsrg_solver_get(const imsrg_solver* solver, const char* name, double* value);
/* IMSRGSolver::SetScratchDir (src/IMSRGSolver.hh:90): when not empty, each
 * Omega finished by an Omega split is written to <dir>/OMEGA_<pid><n> in the
 * reference's binary layout (imsrg_op_write_binary) and its device memory is
 * reused; Transform reads the files back.  A directory containing "/dev/null"
 * counts the Omegas without writing them, as the reference does.  The files
 * are removed when the solver is destroyed.  "" (the default) keeps every
 * Omega in device memory.  imsrg_solver_get reads "n_omega_written". */
int imsrg_solver_set_scratch_dir(imsrg_solver* solver, const char* dir);
/* IMSRGSolver::SetGenerator ("white", "atan", "wegner", "imaginary-time"):
 * starts a new Omega when the current one is not empty (src/IMSRGSolver.cc:157-183). */
int imsrg_solver_set_generator(imsrg_solver* solver, const char* type, void* stream);
/* IMSRGSolver::SetDenominatorPartitioning ("Epstein_Nesbet", "Moller_Plesset") */
int imsrg_solver_set_denominator_partitioning(imsrg_solver* solver, const char* partitioning);
/* IMSRGSolver::Solve() with the solver's method (src/IMSRGSolver.cc:201-504):
 * magnus_euler (the default) flows from the current s to smax or until |eta| <
 * eta_criterion, with IMSRG_ERR_DIVERGED when the reference's give-up test
 * fires (H(s) is then multiplied by 1/0, as there); magnus_modified_euler and
 * magnus_backoff follow Solve_magnus_modified_euler and Solve_magnus_backoff;
 * flow_RK4 follows Solve_flow_RK4 (src/IMSRGSolver.cc:505-636): fixed RK4
 * steps of ds_max on H(s) itself, no Omega. */
int imsrg_solver_solve(imsrg_solver* solver, int precision, void* stream);
/* GetH_s, GetEta and GetOmega(i) (0 <= i < n_omega): the solver's operators */
int imsrg_solver_hs(imsrg_solver* solver, imsrg_op** out);
int imsrg_solver_eta(imsrg_solver* solver, imsrg_op** out);
int imsrg_solver_omega(imsrg_solver* solver, int i, imsrg_op** out);
/* IMSRGSolver::AddOperator / GetOperator (src/IMSRGSolver.hh:94-95): a copy
 * of op (scalar or reduced tensor, of the solver's model space) joins the
 * flowing operators (the copy is complete on return); *index (may be NULL)
 * receives its index.  Operator 0 is
 * H(s).  flow_RK4 flows every added operator with the stage generators of
 * H(s); the Magnus methods leave them as added, as the reference does (their
 * observables go through imsrg_solver_transform). */
int imsrg_solver_add_operator(imsrg_solver* solver, const imsrg_op* op, int* index, void* stream);
int imsrg_solver_get_operator(imsrg_solver* solver, int i, imsrg_op** out);
/* Flow record, one entry per step of every solve (WriteFlowStatus columns,
 * src/IMSRGSolver.cc:1206-1231): step, s, H(s).ZeroBody, |eta| and |Omega|
 * before the step.  Arrays may be NULL; *n receives the number of entries,
 * at most cap are written. */
int imsrg_solver_history(const imsrg_solver* solver, int cap, int* istep, double* s, double* e0, double* norm_eta,
                         double* norm_omega, int* n);
/* IMSRGSolver::Transform (src/IMSRGSolver.cc:928-1002): OpOut = e^Omega OpIn
 * e^-Omega through every Omega in order (scratch files first); InverseTransform
 * (:939-952) undoes the Omegas held in device memory (as the reference, it
 * does not read scratch files).  OpIn and OpOut are scalar or tensor
 * operators of one rank (observables); OpOut may alias OpIn. */
int imsrg_solver_transform(const imsrg_solver* solver, const imsrg_op* OpIn, imsrg_op* OpOut, int precision,
                           void* stream);
int imsrg_solver_inverse_transform(const imsrg_solver* solver, const imsrg_op* OpIn, imsrg_op* OpOut, int precision,
                                   void* stream);

/* ------------------------------------------------------------- profiling */
/* Named phase timers measured with CUDA events on the stream each phase ran
 * on, and a count of kernel launches: the counterpart of IMSRGProfiler's
 * timer / counter maps (src/IMSRGProfiler.cc:14-137; the reference adds each
 * term's wall time under its function name, e.g. src/Commutator.cc:580).
 * Off by default; names are the reference's term names plus kernel phases. */
int imsrg_profiler_enable(int on);
int imsrg_profiler_reset(void);
int imsrg_profiler_get(const char* name, double* total_ms, long long* count);
/* newline-separated timer names; with buf == NULL returns the size needed */
int imsrg_profiler_names(char* buf, int buflen);
long long imsrg_kernel_launches(void);

#ifdef __cplusplus
}
#endif

#endif /* IMSRG_GB300_H */
