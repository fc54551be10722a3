/*
 * qcm_gb300.h -- C ABI of the GB300 two-site SU2U1 DMRG hot path.
 *
 * All entry points are plain C: integer status codes, plain pointers and
 * sizes.  Tensor *layouts* (quantum-number block lists) travel as host
 * arrays; tensor *data* are device pointers to FP64 arrays in which every
 * block is stored column-major (ld = rows) at the element offset given in its
 * layout, blocks in the reference's DualIndex order (descending on the
 * (left, right) charge pair).  A charge is the pair (N, 2S).
 *
 * The reference interfaces these entry points replace (paths relative to the
 * QCMaquis source tree):
 *   contraction::Engine<..., SU2>::site_hamil2
 *       dmrg/framework/dmrg/mp_tensors/contractions/non-abelian/engine.hpp:197-207
 *       -> qcm_plan_sigma + qcm_plan_run
 *   contraction::Engine<..., SU2>::overlap_mpo_left_step
 *       .../non-abelian/engine.hpp:104-113 -> qcm_plan_boundary_left + qcm_plan_run
 *   contraction::Engine<..., SU2>::overlap_mpo_right_step
 *       .../non-abelian/engine.hpp:115-124 -> qcm_plan_boundary_right + qcm_plan_run
 *   contraction::Engine<..., SU2>::left/right_boundary_tensor_mpo
 *       .../non-abelian/engine.hpp:84-102 -> qcm_plan_boundary_tensor_mpo + qcm_plan_run
 *   ietl::dot / ietl::two_norm on MPSTensor (scalar_overlap, norm)
 *       dmrg/framework/dmrg/mp_tensors/mpstensor.hpp:365-380 -> qcm_dot, qcm_nrm2
 *   vector updates inside jacobi_davidson::calculate_eigenvalue
 *       dmrg/framework/ietl/jacobi.h:385-435 -> qcm_axpby
 *
 * Error behaviour: every call returns QCM_OK (0) or a negative QCM_E_* code;
 * qcm_last_error() returns a message for the calling thread.  The reference
 * throws std::runtime_error in the same situations.
 */
#ifndef QCM_GB300_H
#define QCM_GB300_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define QCM_OK 0
#define QCM_E_INVALID (-1)   /* malformed layout / MPO / argument */
#define QCM_E_CUDA (-2)      /* a CUDA runtime call failed */
#define QCM_E_NOMEM (-3)     /* device allocation failed */
#define QCM_E_STATE (-4)     /* plan not uploaded / wrong plan kind */
#define QCM_E_RANGE (-5)     /* request exceeds a fixed capacity */

/* Quantum-number index: n sectors, charges q[2*i], q[2*i+1] = (N, 2S), sizes. */
typedef struct {
    int32_t n;
    const int32_t* q;
    const int64_t* size;
} qcm_index_t;

/* Block list of one block-sparse matrix.
 * q[4*k..4*k+3] = (lc.N, lc.2S, rc.N, rc.2S); off[k] = element offset. */
typedef struct {
    int32_t n;
    const int32_t* q;
    const int64_t* rows;
    const int64_t* cols;
    const int64_t* off;
} qcm_blocks_t;

/* Boundary = one block matrix per MPO bond index b (mp_tensors/boundary.h:20-145).
 * Blocks of b occupy [blk_ptr[b], blk_ptr[b+1]) of the flattened arrays;
 * offsets index one arena holding all b. */
typedef struct {
    int32_t aux;
    const int32_t* blk_ptr;
    const int32_t* q;
    const int64_t* rows;
    const int64_t* cols;
    const int64_t* off;
} qcm_boundary_t;

/* MPO tensor (mp_tensors/mpotensor.h:23-107) flattened.
 * Elements (b1,b2) are listed column by column: column b2 owns
 * [col_ptr[b2], col_ptr[b2+1]); row_of[e] = b1; its (op, scale) terms are
 * [term_ptr[e], term_ptr[e+1]).  Operator o has SU(2) rank op_spin[o] and
 * blocks [op_blk_ptr[o], op_blk_ptr[o+1]); block k maps phys charge
 * (blk_q[4k], blk_q[4k+1]) to (blk_q[4k+2], blk_q[4k+3]) and owns sparse
 * entries [blk_ent_ptr[k], blk_ent_ptr[k+1]) with ent[4e..4e+3] =
 * (row, col, row_spin, col_spin) and value ent_coeff[e]
 * (block_matrix/sparse_operator.h:105-168).  Hermitian data follow
 * mp_tensors/mpotensor_detail.h:124-160 (partner index and phase).
 * symmetry selects the group of the charges (QCM_SYM_*): SU2U1 charges are
 * (N, 2S) and the contractions carry the SU(2) couplings (ct/non-abelian);
 * TwoU1 charges are (N_up, N_down), every coupling is 1, spins and phases are
 * ignored (ct/abelian); U1 charges are (N, 0) -- the reference's single int
 * charge (block_matrix/symmetry/u1.h) in the first component, the second held at
 * zero, so blocks sort as the reference's U1 blocks do -- and contract as TwoU1.
 * A zero-initialised field means SU2U1. */
typedef struct {
    int32_t row_dim, col_dim;
    const int32_t* left_spin;
    const int32_t* right_spin;
    const int32_t* left_herm;
    const int32_t* right_herm;
    const int32_t* left_phase;
    const int32_t* right_phase;
    const int32_t* col_ptr;
    const int32_t* row_of;
    const int32_t* term_ptr;
    const int32_t* term_op;
    const double* term_scale;
    int32_t n_ops;
    const int32_t* op_spin;
    const int32_t* op_blk_ptr;
    const int32_t* blk_q;
    const int32_t* blk_ent_ptr;
    const int32_t* ent;
    const double* ent_coeff;
    int32_t symmetry;
} qcm_mpo_t;

#define QCM_SYM_SU2U1 0
#define QCM_SYM_TWOU1 1
#define QCM_SYM_U1 2

typedef struct qcm_plan qcm_plan;

/* Buffer slots a plan reads and writes. */
enum {
    QCM_BUF_KET = 0,     /* input MPS tensor data (left-paired layout) */
    QCM_BUF_LEFT = 1,    /* left boundary arena */
    QCM_BUF_RIGHT = 2,   /* right boundary arena */
    QCM_BUF_OUT = 3,     /* output: sigma (ket layout) or new boundary arena */
    QCM_BUF_S0 = 4,      /* scratch 0 */
    QCM_BUF_S1 = 5,      /* scratch 1 */
    QCM_BUF_S2 = 6,      /* scratch 2 */
    QCM_BUF_IMG = 7,     /* operand images of the BF16x3 form (qcm_plan_image_bytes); may be NULL */
    QCM_NBUF = 8
};

/* Precision of the dense block products of a plan. */
enum {
    QCM_PREC_FP64 = 0,      /* all arithmetic FP64 */
    QCM_PREC_TF32 = 1,      /* tcgen05 kind::tf32 products, FP32 accumulation */
    QCM_PREC_BF16X3 = 2,    /* 3-slice BF16 split products, FP32 accumulation */
    QCM_PREC_BF16X2 = 3     /* the same images, the 3 products a_i b_j with i + j <= 1 (2-slice
                               accuracy, half the tensor-core work); image slot required */
};

const char* qcm_last_error(void);
int qcm_version(void);

/* sigma = H_eff psi for a two-site (reduced) tensor; bra = ket.
 * psi/sigma layout: left-paired blocks of the ket.  hermitian != 0 uses the
 * MPO's Hermitian partners (boundaries then hold no blocks at skipped b). */
int qcm_plan_sigma(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                   const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                   const qcm_mpo_t* mpo, int32_t hermitian, qcm_plan** plan);

/* Plan-shape options of a sigma plan (0 = default).  split_k_segs: the largest
 * number of block products summed into one K3 output before it is split into
 * partial tiles (default 32); dense_min_terms: the fewest K2 terms an output tile
 * needs to join a dense tensor-core group (default 64); n_tile_max: the widest N
 * of a tensor-core tile of the block products (16..128 in steps of 16, default
 * 128; wider blocks are cut into tiles of balanced width); k1_schedule: how the
 * K1 tiles go to the CTAs of the persistent image executor (0 = round robin, the
 * default; 1 = contiguous cost-balanced ranges with each A tile kept in shared
 * memory while its tiles run, where every K1 tile is one short block product).
 * Chosen per problem shape by the autotuner of the Python layer
 * (qcmaquis_gb300/autotune.py). */
typedef struct {
    int32_t split_k_segs;
    int32_t dense_min_terms;
    int32_t n_tile_max;
    int32_t k1_schedule;
    int32_t reserved[4];
} qcm_plan_opts_t;

/* qcm_plan_sigma with plan-shape options (NULL: the defaults). */
int qcm_plan_sigma_opts(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                        const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                        const qcm_mpo_t* mpo, int32_t hermitian, const qcm_plan_opts_t* opts, qcm_plan** plan);

/* New left boundary L[i+1] from L[i], site tensor (bra = ket, left-paired) and W[i]. */
int qcm_plan_boundary_left(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                           const qcm_blocks_t* mps, const qcm_boundary_t* left, const qcm_mpo_t* mpo,
                           int32_t hermitian, qcm_plan** plan);

/* New right boundary R[i] from R[i+1], site tensor (left-paired) and W[i]. */
int qcm_plan_boundary_right(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                            const qcm_blocks_t* mps, const qcm_boundary_t* right, const qcm_mpo_t* mpo,
                            int32_t hermitian, qcm_plan** plan);

/* The boundary x MPS x MPO contraction without the bra, one block matrix per
 * MPO bond on the open side (side 0: Engine::left_boundary_tensor_mpo, a
 * block matrix per right bond b2; side 1: right_boundary_tensor_mpo, one per
 * left bond b1; dmrg/framework/dmrg/mp_tensors/contractions/common/
 * move_boundary.hpp:66-126).  Every bond is computed; hermitian != 0 lets the
 * boundary product read the Hermitian partners, as the reference's default.
 * Output layout through qcm_plan_out_layout.  Its use in the reference is the
 * density-matrix perturbation of the heev truncation
 * (mp_tensors/twositetensor.hpp:184-297), with the two-site tensor seen as
 * one site (side 0: physical index of site 1, right index adjoin(phys2) x
 * right; side 1: physical index of site 2, left index phys1 x left). */
int qcm_plan_boundary_tensor_mpo(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                                 const qcm_blocks_t* mps, const qcm_boundary_t* boundary, const qcm_mpo_t* mpo,
                                 int32_t side, int32_t hermitian, qcm_plan** plan);

/* Two-site MPO tensor on the host (make_twosite_mpo, dmrg/framework/dmrg/
 * mp_tensors/ts_ops.h:78-152): W(b1,b3) = sum_b2 W1(b1,b2) (x) W2(b2,b3), one
 * operator per allowed product spin s, flattened as qcm_mpo_t.  Three steps:
 * qcm_mpo_twosite_begin walks the non-zero (b1, b2, b3) chains and returns the
 * number of distinct spin-coupled Kronecker products they need;
 * qcm_mpo_twosite_keys lists them, 6 int32 each: (operator of W1, operator of
 * W2, spin of b1, spin of b2, spin of b3, s); the caller forms each product
 * (SU(2) op_kron, site_operator_algorithms.h) and passes them, in key order, as
 * the operators of a qcm_mpo_t -- n_ops, op_spin, op_blk_ptr, blk_q, blk_ent_ptr,
 * ent, ent_coeff; the other fields are not read -- to qcm_mpo_twosite_finish,
 * which sums the scaled products of every (b1, b3, s) in the reference's order.
 * qcm_mpo_buf_view points a qcm_mpo_t at the result (valid until
 * qcm_mpo_buf_destroy); sizes[4] = elements, terms, operator blocks, entries.
 * Terms are listed element by element, column-major; an element's operators
 * with s descending; qcm_mpo_buf_term_pos gives each term's position in its
 * element.  Every term has scale 1 and its own operator. */
typedef struct qcm_mpo_buf qcm_mpo_buf;
int qcm_mpo_twosite_begin(const qcm_mpo_t* w1, const qcm_mpo_t* w2, qcm_mpo_buf** out, int32_t* n_keys);
int qcm_mpo_twosite_keys(const qcm_mpo_buf* buf, int32_t* keys);
int qcm_mpo_twosite_finish(qcm_mpo_buf* buf, const qcm_mpo_t* products);
int qcm_mpo_buf_view(const qcm_mpo_buf* buf, qcm_mpo_t* view, int64_t* sizes);
int qcm_mpo_buf_term_pos(const qcm_mpo_buf* buf, int32_t* pos);
void qcm_mpo_buf_destroy(qcm_mpo_buf* buf);
/* The three steps in one call, the SU(2) op_kron (site_operator_algorithms.h) in
 * native code too: phys1, phys2 are the two sites' local indices.  Its Wigner
 * symbols are long-double Racah sums, so coefficients can differ from an
 * exact-rational evaluation in the last bits.  View and destroy as above. */
int qcm_mpo_twosite(const qcm_mpo_t* w1, const qcm_mpo_t* w2, const qcm_index_t* phys1, const qcm_index_t* phys2,
                    qcm_mpo_buf** out);

/* Single-site MPO tensors from the model's terms (TaggedMPOMaker,
 * dmrg/framework/dmrg/models/generate_mpo/tagged_mpo_maker_optim.hpp:
 * add_term / add_generic_term with their fork keys and filling strings,
 * :168-187, :472-560, :594-638; finalize, :640-669; create_mpo with the bond
 * numbering in key order, the bond spins and the Hermitian bond pairs, :189-300,
 * with the phases of conjugate_key, :671-735).
 *
 * The tag table describes the operators the terms name: per tag whether it is
 * fermionic, its spin (2S, action) -- two int32 per tag --, its Hermitian
 * conjugate tag and pdiff = N(in) - N(out) of its first block (the particle
 * number change the SU(2) bond phases read); and the tags of the identity, the
 * identity of spin > 1 bonds and the fermionic filling.
 *
 * qcm_mpo_maker_add_terms takes terms of two or more operators, CSR style
 * (term t = positions/tags [term_ptr[t], term_ptr[t+1]), sorted by position
 * inside the call, stable), with the coefficient on the operator the reference
 * attaches it to and a caller label per term (-1: none) carried to that scale.
 * One-site terms are the caller's (they need its operator algebra): it passes
 * each site's (TL, TR) element list to qcm_mpo_maker_site_terms, then
 * qcm_mpo_maker_finish with the final tag table (site operators registered
 * since create added), the smallest last position and the largest first
 * position over all terms (one-site terms included).  qcm_mpo_maker_site views
 * one site's tensor, valid until qcm_mpo_maker_destroy: elements column-major,
 * each element's (tag, scale, label) terms in the reference's MPOTensor order
 * (latest insertion first), the outgoing bonds' spins (2S, action), Hermitian
 * partners and phases (bond_dim entries; the incoming bonds' are the previous
 * site's).  row_dim / col_dim are 1 at the chain ends.  A maker is finished once:
 * after a failed qcm_mpo_maker_finish it refuses further calls (QCM_E_STATE) and
 * is only destroyed. */
typedef struct {
    int32_t n_tags;
    const int32_t* fermionic;  /* n_tags */
    const int32_t* spin;       /* 2 * n_tags: (2S, action) */
    const int32_t* herm_conj;  /* n_tags */
    const int32_t* pdiff;      /* n_tags */
    int32_t identity, identity_full, fill;
    int32_t symmetry;          /* QCM_SYM_*: abelian groups pair bonds with phase 1 */
} qcm_tag_table_t;

typedef struct {
    int32_t row_dim, col_dim, bond_dim;
    int32_t n_elem;
    const int32_t* elem_b1;    /* n_elem */
    const int32_t* elem_b2;    /* n_elem */
    const int32_t* elem_ptr;   /* n_elem + 1, into the term arrays */
    const int32_t* term_tag;
    const double* term_scale;
    const int32_t* term_label;
    const int32_t* right_spin; /* 2 * bond_dim */
    const int32_t* right_herm; /* bond_dim */
    const int32_t* right_phase;/* bond_dim */
} qcm_mpo_site_t;

/* Terms of the SU2U1 quantum-chemistry Hamiltonian (qc_su2 model,
 * dmrg/framework/dmrg/models/chem/su2u1/model.hpp:52-203, with the SU(2) term
 * makers and spin sums of models/chem/su2u1/term_maker.h:120-395, :548-793): the
 * n_int integrals (idx: four 1-based orbital indices each, 0 = unused, as in
 * the reference's integral map; val: their values; |val| <= cutoff skipped)
 * become operator terms.  One-site terms come first in integral order; the
 * two-, three- and four-operator terms follow, equal terms merged (coefficients
 * summed), in ascending order of (positions, tags).  Off-diagonal one-body
 * integrals are folded into two-body terms with weight 1/(nelec-1)
 * (model.hpp:96-139).  Each term lists, per integral it came from (index into
 * the input), its coefficient per unit of that integral.  The tag table names
 * the model's operators: bundles[b][f] for b = create, destroy, count, flip,
 * e2d, d2e, docc, create_count, destroy_count and f = couple_up, couple_down,
 * fill_couple_up, fill_couple_down, no_couple, fill_no_couple (-1 where a
 * bundle has no such operator). */
typedef struct {
    int32_t ident, count, docc;
    int32_t bundles[9][6];
} qcm_chem_tags_t;

typedef struct {
    int64_t n_terms;
    const int32_t* term_ptr;   /* n_terms + 1, into pos / tag */
    const int32_t* pos;
    const int32_t* tag;
    const double* coeff;       /* n_terms */
    const int32_t* fermionic;  /* n_terms */
    const int64_t* src_ptr;    /* n_terms + 1, into src_idx / src_val */
    const int64_t* src_idx;    /* integral index */
    const double* src_val;     /* coefficient per unit of that integral */
} qcm_term_view_t;

typedef struct qcm_term_buf qcm_term_buf;
int qcm_chem_terms(int32_t L, int32_t nelec, int64_t n_int, const int32_t* idx, const double* val, double cutoff,
                   const qcm_chem_tags_t* tags, qcm_term_buf** out);
int qcm_term_buf_view(const qcm_term_buf* buf, qcm_term_view_t* view);
void qcm_term_buf_destroy(qcm_term_buf* buf);

typedef struct qcm_mpo_maker qcm_mpo_maker;
int qcm_mpo_maker_create(int32_t L, const qcm_tag_table_t* tags, qcm_mpo_maker** out);
int qcm_mpo_maker_add_terms(qcm_mpo_maker* maker, int32_t n_terms, const int32_t* term_ptr, const int32_t* pos,
                            const int32_t* tag, const double* coeff, const int32_t* label);
int qcm_mpo_maker_site_terms(qcm_mpo_maker* maker, int32_t site, int32_t n, const int32_t* tag, const double* scale,
                             const int32_t* label);
int qcm_mpo_maker_finish(qcm_mpo_maker* maker, const qcm_tag_table_t* tags, int32_t leftmost_right,
                         int32_t rightmost_left);
int qcm_mpo_maker_site(const qcm_mpo_maker* maker, int32_t site, qcm_mpo_site_t* view);
void qcm_mpo_maker_destroy(qcm_mpo_maker* maker);

/* Diagonal of H_eff (Engine::diagonal_hamiltonian, dmrg/framework/dmrg/mp_tensors/
 * contractions/non-abelian/engine.hpp:221-226 -> SU2::diagonal_hamiltonian,
 * non-abelian/h_diag.hpp:118-158), the arguments of qcm_plan_sigma without
 * hermitian: every L[b1] and R[b2] is read as given, so the boundaries must hold
 * every bond index (built with hermitian = 0).  OUT has psi's layout.  FP64 form
 * only (other precisions: QCM_E_INVALID). */
int qcm_plan_diagonal(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                      const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                      const qcm_mpo_t* mpo, qcm_plan** plan);

/* Zero-site problem (ZeroSiteProblem::apply, dmrg/framework/dmrg/mp_tensors/
 * zerositeproblem.h:40-42 -> zerosite_hamil_lbtm_kernel, dmrg/framework/dmrg/
 * mp_tensors/contractions/non-abelian/zero_site_hamil.hpp:44-79): sigma =
 * H_eff C for the bond matrix C between sites i and i+1 (block diagonal in the
 * bond's charges), with left = L[i+1], right = R[i+1], mpo_left = W[i] (its
 * columns are the bond) and mpo_right = W[i+1] (its rows are the bond).  sigma
 * has C's layout; the plan's KET buffer is C.  hermitian != 0 uses the bond's
 * Hermitian partners, without phases, as the reference does. */
int qcm_plan_zerosite(const qcm_blocks_t* bond, const qcm_boundary_t* left, const qcm_boundary_t* right,
                      const qcm_mpo_t* mpo_left, const qcm_mpo_t* mpo_right, int32_t hermitian, qcm_plan** plan);

/* Gradient of the local energy E = <psi| H_eff psi> (the contraction of
 * qcm_plan_sigma, same arguments) with respect to every term scale of the MPO
 * tensor: OUT[t] = dE/d term_scale[t], t indexing the flattened term arrays of
 * qcm_mpo_t; out_elems is their length.  With left = L[j], right = R[j+1] and
 * psi = the site tensor of a single-site problem at j, E is <Psi|H|Psi> of the
 * whole MPS, so OUT is the derivative of the energy expectation value with
 * respect to the site-j MPO coefficients -- the adjoint behind dE/d(t_pq),
 * dE/d(V_pqrs) and the RDMs.  Stages: K1, the adjoint of K3 (Y = dE/dcontr,
 * grouped GEMM), per-term dots of the K2 tables against Y and their sums per
 * term scale.  FP64 form only (other precisions: QCM_E_INVALID).  Not a
 * reference entry point: the reference obtains RDMs by separate expectation
 * values (dmrg/framework/dmrg/models/measurements/tagged_nrankrdm_su2u1.h). */
int qcm_plan_energy_gradient(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                             const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                             const qcm_mpo_t* mpo, int32_t hermitian, qcm_plan** plan);

/* Batching: one plan for n independent sigma problems (plans of qcm_plan_sigma).
 * caller_off holds, per problem, the element offsets of its KET, LEFT, RIGHT and
 * OUT data inside the buffers passed to qcm_plan_run (4 per problem); the scratch
 * slots and the operand images of the problems are laid out back to back by the
 * merged plan (qcm_plan_sizes, qcm_plan_image_bytes).  Each stage of the merged
 * plan runs every problem's work in one launch: one persistent grouped block-
 * product launch per stage for all problems.  The sub-plans stay valid. */
int qcm_plan_merge(qcm_plan* const* plans, int32_t n, const int64_t* caller_off, qcm_plan** out);

/* Sizes (elements) of the output and of the three scratch slots. */
int qcm_plan_sizes(const qcm_plan* plan, int64_t* out_elems, int64_t* scratch_elems3);

/* Bytes of the operand-image buffer (slot QCM_BUF_IMG) that the BF16x3 form
 * uses to feed its block products to the tensor cores by bulk copies.  When
 * that slot is NULL the BF16x3 form splits operands inside its block-product
 * kernel instead (same results, slower). */
int qcm_plan_image_bytes(const qcm_plan* plan, int64_t* bytes);

/* Number of kernels the plan's last run launched (memsets excluded): the
 * executors chosen depend on the precision and on the image buffer. */
int qcm_plan_last_kernels(const qcm_plan* plan, int32_t* n);

/* Work counters: algorithmic FLOPs of the block products, FLOPs and bytes of the
 * gather/axpy stages, and the number of kernel launches of one run. */
int qcm_plan_work(const qcm_plan* plan, double* gemm_flops, double* axpy_flops, double* axpy_bytes,
                  int32_t* launches);

/* Output boundary layout of a boundary plan (aux, then per-block arrays of
 * length nblocks).  Call first with NULL arrays to get aux and nblocks. */
int qcm_plan_out_layout(const qcm_plan* plan, int32_t* aux, int32_t* nblocks, int32_t* blk_ptr,
                        int32_t* q, int64_t* rows, int64_t* cols, int64_t* off);

/* Stage export for host-side inspection: kind 0 = gather-axpy, 1 = grouped GEMM,
 * 2 = clear (n_out = slot, n_terms = length), 3 = per-term dots of an energy-gradient plan. */
int qcm_plan_num_stages(const qcm_plan* plan, int32_t* n);
int qcm_plan_stage_info(const qcm_plan* plan, int32_t stage, int32_t* kind, int64_t* n_out, int64_t* n_terms);
int qcm_plan_stage_axpy(const qcm_plan* plan, int32_t stage, int64_t* out_desc /*7*n_out*/,
                        int64_t* term_desc /*3*n_terms*/, double* term_alpha);
int qcm_plan_stage_gemm(const qcm_plan* plan, int32_t stage, int64_t* out_desc /*7*n_out*/,
                        int64_t* seg_desc /*9*n_terms*/, double* seg_alpha);
/* Dot stage: output-adjoint tiles (7 per tile, as qcm_plan_stage_axpy), terms
 * (3 each), per-term weight and MPO term index; meta = {dot buffer slot, number
 * of MPO terms}. */
int qcm_plan_stage_dot(const qcm_plan* plan, int32_t stage, int64_t* out_desc, int64_t* term_desc, double* weight,
                       int32_t* term_index, int32_t* meta);

/* Export the BF16x3 image-executor tables of a stage (host-side inspection
 * and tests): the block products of a GEMM stage, or the dense groups of a
 * gather-axpy stage.  counts4 = (panels, outputs, segments, tiles); call with
 * NULL arrays first.  panel: (src_off, img_off, src_buf, ld, R, K, kcontig, G);
 * output: (c_off, si, sj, c_buf, mrows, ncols, mode, rows, ctab, vrows) -- for
 * mode 1 with vrows > 0 each column is a run of pitch `rows` of which the first
 * vrows rows are stored; segment:
 * (a_img, b_img, a_G, b_G, kc, flags, a_panel, a_c0) with seg_alpha; tile:
 * (out, m0, n0, nt, s_begin, s_end).  A panel without an image has img_off -1. */
int qcm_plan_stage_images(const qcm_plan* plan, int32_t stage, int64_t* counts4, int64_t* panel_desc /*8*n*/,
                          int64_t* out_desc /*10*n*/, int64_t* seg_desc /*8*n*/, double* seg_alpha,
                          int64_t* tile_desc /*6*n*/);
/* Auxiliary tables of the same: counts3 = (gather offsets, output-tile
 * offsets, constant-image bytes). */
int qcm_plan_stage_image_aux(const qcm_plan* plan, int32_t stage, int64_t* counts3, int64_t* gather,
                             int64_t* coltab, uint8_t* const_images);

/* Copy the plan's task tables to the current device (once per plan). */
int qcm_plan_upload(qcm_plan* plan);

/* Run the plan on a CUDA stream (NULL = default stream); bufs[QCM_NBUF] are
 * device pointers.  precision selects FP64 or a tensor-core form. */
int qcm_plan_run(qcm_plan* plan, double* const* bufs, int32_t precision, void* stream);

/* Run only stages [first, last] (last < 0: through the final stage); used to
 * time individual kernels.  Stage kinds are reported by qcm_plan_stage_info. */
int qcm_plan_run_stages(qcm_plan* plan, double* const* bufs, int32_t precision, void* stream, int32_t first,
                        int32_t last);

/* Run with explicit element types: bit i of f32mask marks buffer slot i as FP32.
 * The FP64 form requires f32mask == 0.  The mixed forms accept FP32 or FP64 for
 * every slot; qcm_plan_run uses FP32 scratch and FP64 caller slots, and callers
 * that keep FP32 copies of the boundaries set the LEFT/RIGHT bits as well. */
int qcm_plan_run_typed(qcm_plan* plan, double* const* bufs, uint32_t f32mask, int32_t precision, void* stream,
                       int32_t first, int32_t last);

void qcm_plan_destroy(qcm_plan* plan);

/* Sticky status word of the tensor-core executor: 0 = ok, 1 = a bounded wait
 * for tensor-core completion timed out (the kernel released its TMEM and
 * returned without writing its tile). */
int qcm_device_status(int32_t* status);

/* FP64 vector kernels over n elements (deterministic reductions).
 * The result of qcm_dot / qcm_nrm2 is written to a device double.
 * qcm_dot, qcm_nrm2 and qcm_multi_dot share one library-owned workspace per
 * device (partial sums and a vector-pointer table, allocated on first use):
 * calls issued on streams with no ordering between them race on it, so issue
 * them on one stream (or order the streams). */
int qcm_dot(const double* x, const double* y, int64_t n, double* result_dev, void* stream);
int qcm_nrm2(const double* x, int64_t n, double* result_dev, void* stream);
/* y = a*x + b*y */
int qcm_axpby(double a, const double* x, double b, double* y, int64_t n, void* stream);
/* y[i] = sum_k coef[k] * X[k][i]  for k < nvec (coef on the host) */
int qcm_lincomb(const double* const* x_dev_ptrs, const double* coef, int32_t nvec, double* y, int64_t n,
                void* stream);
/* out[k] = dot(V_k, y) for k < nvec, results in a device array of nvec doubles */
int qcm_multi_dot(const double* const* v_dev_ptrs, int32_t nvec, const double* y, int64_t n, double* out_dev,
                  void* stream);

/* Allocation-free variant of qcm_multi_dot.  No counterpart in the reference:
 * it exists for callers that cannot allocate device memory during a solve --
 * hosts that hand the whole device budget to their own memory pool up front
 * and forbid cudaMalloc afterwards (an allocation there would synchronise the
 * device and break the pool's accounting).  It computes the same
 * out[k] = dot(V_k, y) with the same reduction order as qcm_multi_dot, but its
 * partial sums live in a fixed library-owned device array of 32 x 304 doubles
 * instead of a workspace allocated on first use; every GPU that loads the
 * library holds that array until the process exits.
 * Limits: nvec <= 32, otherwise QCM_E_RANGE and nothing is launched.
 * The first call on each device looks up the array's device address and,
 * with CUDA's default lazy module loading, may load the library's device code,
 * which takes device memory for the code and the array: make that first call
 * before the host's pool reserves the device budget (or run with
 * CUDA_MODULE_LOADING=EAGER) and before any stream capture.  All calls share the array:
 * calls that overlap on the GPU (different streams, no ordering between them)
 * race on it and must be serialised by the caller. */
int qcm_multi_dot_noalloc(const double* const* v_dev_ptrs, int32_t nvec, const double* y, int64_t n,
                          double* out_dev, void* stream);

/* Segmented dots for eigensolvers that run several problems in lockstep on
 * concatenated vectors: out_dev[j * nseg + k] = sum over i in [seg_off[k],
 * seg_off[k+1]) of V_j[i] * y[i], for j < nvec (<= 32) and k < nseg.  seg_off is a
 * device array of nseg + 1 element offsets; v_dev_ptrs is a host array of device
 * pointers.  Fixed reduction order; allocates nothing. */
int qcm_seg_multi_dot(const double* const* v_dev_ptrs, int32_t nvec, const double* y, const int64_t* seg_off_dev,
                      int32_t nseg, double* out_dev, void* stream);

/* Truncation results (truncation_results, dmrg/framework/dmrg/block_matrix/
 * block_matrix_algorithms.h:211-333). */
typedef struct {
    int64_t bond_dimension;
    double truncated_weight;
    double truncated_fraction;
    double smallest_ev;
    double evalscut;
} qcm_trunc_t;

/* ---------------------------------------------------------------- execution context
 * A context owns what plan runs need besides the caller's tensors: its CUDA
 * stream, the plans' scratch slots and operand-image buffer, FP32 shadows of
 * the boundaries for the mixed forms, and the eigensolver's basis vectors and
 * reduction workspace (SURVEY's proposed qcm_ctx; the reference has no
 * counterpart -- its Engine calls allocate per call).  Its device buffers grow
 * on demand and are freed by qcm_ctx_destroy.  Calls on one context run in
 * order on its stream and are not reentrant; different contexts share nothing.
 * Created on the current device. */
typedef struct qcm_ctx qcm_ctx;
int qcm_ctx_create(void* stream, qcm_ctx** ctx);
int qcm_ctx_set_stream(qcm_ctx* ctx, void* stream);
void qcm_ctx_destroy(qcm_ctx* ctx);

/* Run any plan with the context's scratch: ket/left/right/out fill the KET,
 * LEFT, RIGHT and OUT slots (FP64 device arrays; NULL where the plan reads
 * none).  The mixed forms convert left/right (left_elems / right_elems
 * doubles) to FP32 shadows first. */
int qcm_ctx_run(qcm_ctx* ctx, qcm_plan* plan, const double* ket, const double* left, int64_t left_elems,
                const double* right, int64_t right_elems, double* out, int32_t precision);

/* One boundary update (BoundaryPropagator::updateLeftBoundary / updateRightBoundary,
 * dmrg/framework/dmrg/SweepBasedAlgorithms/BoundaryPropagator.h:98-122 ->
 * overlap_mpo_left_step / overlap_mpo_right_step): a plan of
 * qcm_plan_boundary_left / _right run on the context; boundary is L[i] (left)
 * or R[i+1] (right), out the new boundary (qcm_plan_out_layout). */
int qcm_boundary_step(qcm_ctx* ctx, qcm_plan* plan, const double* mps, const double* boundary, int64_t boundary_elems,
                      double* out, int32_t precision);

/* Jacobi-Davidson eigensolver of one site problem (solve_ietl_jcd,
 * dmrg/framework/dmrg/optimize/ietl_jacobi_davidson.h:16-77, with
 * jacobi_davidson::calculate_eigenvalue, dmrg/framework/ietl/jacobi.h:361-451,
 * zero GMRES steps as on the reference's live path): the smallest eigenpair of
 * H_eff = the sigma plan on (left, right) in the given precision, from init (n
 * doubles, the plan's ket layout), stopping when |r| <= tol |theta|, |r| < tol
 * or after maxiter (<= 32) steps.  ortho: device vectors the solution is kept
 * orthogonal to (excited states; <= 16).  Writes the eigenvector to out_vec
 * (device), the eigenvalue and the iterations to the host.  Vector algebra
 * and Gram-Schmidt run in FP64 on the context's stream; two host
 * synchronisations per iteration (projected-matrix column, residual norm). */
int qcm_jcd_solve(qcm_ctx* ctx, qcm_plan* sigma, const double* left, int64_t left_elems, const double* right,
                  int64_t right_elems, int32_t precision, const double* init, int64_t n, double tol, int32_t maxiter,
                  const double* const* ortho, int32_t n_ortho, double* out_vec, double* out_energy,
                  int32_t* out_iters);

/* TwoSiteTensor::split_mps_l2r / split_mps_r2l (dmrg/framework/dmrg/mp_tensors/
 * twositetensor.hpp:141-180, with svd_truncate, dmrg/framework/dmrg/
 * block_matrix/block_matrix_algorithms.h:163-333) of the reduced two-site
 * tensor u (layout u, data u_dev; phys1/phys2 the sites' physical indices,
 * left_i / right_i the pair's outer indices), entirely on the device: the
 * split-prologue plan, the batched Jacobi SVD of the both-paired blocks, the
 * device cut (Mmax, cutoff) and the assembly plan.  l2r != 0: A = U, B = S V;
 * else A = U S, B = V.  The new site tensors (left-paired, with their indices)
 * are owned by the result (qcm_split_result_tensor: which 0 = site i, 1 = site
 * i+1; the same arrays as qcm_plan_out_tensor plus the device data pointer,
 * valid until qcm_split_result_destroy); trunc receives bond dimension,
 * truncated weight and fraction, and smallest_ev as the reference reports
 * them.  symmetry (QCM_SYM_*) as for qcm_plan_split_theta.  Synchronises the
 * context's stream. */
typedef struct qcm_split_result qcm_split_result;
int qcm_split(qcm_ctx* ctx, const qcm_index_t* phys1, const qcm_index_t* phys2, const qcm_index_t* left_i,
              const qcm_index_t* right_i, const qcm_blocks_t* u, const double* u_dev, int32_t l2r, int64_t Mmax,
              double cutoff, int32_t symmetry, qcm_trunc_t* trunc, qcm_split_result** out);
int qcm_split_result_tensor(const qcm_split_result* res, int32_t which, int32_t* nblocks, int32_t* q, int64_t* rows,
                            int64_t* cols, int64_t* off, int32_t* n_idx3, int32_t* idx_q, int64_t* idx_size,
                            const double** data);
void qcm_split_result_destroy(qcm_split_result* res);

/* ---------------------------------------------------------------- MPS-level steps
 * The linear maps around the eigensolver as plans (qcm_plan_upload /
 * qcm_plan_run, FP64): every map is planned once as gather tiles with its
 * couplings precomputed, and runs as one gather launch; nothing is done per
 * block on the host.
 *
 * TwoSiteTensor(mps1, mps2) + make_mps (dmrg/framework/dmrg/mp_tensors/
 * twositetensor.hpp:22-31, 132-139): theta = A . B, reshape_both_to_right,
 * the SU(2) reduce_right 6j recoupling (mp_tensors/ts_reduction.h:42-141) and
 * the reshape to left-paired.  Slots: KET = A (left-paired), LEFT = B
 * (left-paired), OUT = the reduced two-site tensor; its layout and indices
 * through qcm_plan_out_tensor.  With symmetry = QCM_SYM_TWOU1 there is no
 * reduction: the two-site physical index is the product phys1 x phys2 and the
 * tensor is reshaped straight to left-paired (make_mps_ of the abelian
 * TwoSiteTensor, twositetensor.hpp:125-130); QCM_SYM_U1 likewise. */
int qcm_plan_two_site(const qcm_index_t* phys1, const qcm_index_t* a_left, const qcm_index_t* a_right,
                      const qcm_blocks_t* a, const qcm_index_t* phys2, const qcm_index_t* b_left,
                      const qcm_index_t* b_right, const qcm_blocks_t* b, int32_t symmetry, qcm_plan** plan);

/* The prologue of split_mps_l2r/r2l (twositetensor.hpp:141-180 with operator<<,
 * :372-389): the SU(2) unreduce_left recoupling (ts_reduction.h:143-251) and
 * reshape_left_to_both.  left_i / right_i are the outer indices of the pair
 * (left of site i, right of site i+1).  Slots: KET = the reduced two-site
 * tensor (left-paired), OUT = the both-paired matrix the truncation factorises
 * (its blocks through qcm_plan_out_tensor; they are the qcm_svd batch).
 * QCM_SYM_TWOU1 and QCM_SYM_U1: no unreduce step (the abelian operator<<,
 * twositetensor.hpp:352-366), only the reshape. */
int qcm_plan_split_theta(const qcm_index_t* phys1, const qcm_index_t* phys2, const qcm_index_t* left_i,
                         const qcm_index_t* right_i, const qcm_blocks_t* u, int32_t symmetry, qcm_plan** plan);

/* The epilogue of split_mps_l2r (l2r != 0: A = U, B = S V) or split_mps_r2l
 * (A = U S, B = V), after the truncation cut: from the qcm_svd of the split
 * plan's output blocks (u_off, vt_off, s_off from qcm_svd_block_offsets; S on
 * the host; keep[k] from qcm_truncation_cut).  Slots: KET = U, LEFT = Vt; OUT =
 * the new site i (left-paired, qcm_plan_out_tensor which = 0), S2 = the new
 * site i+1 (left-paired, which = 1); S0 is scratch. */
int qcm_plan_split_assemble(const qcm_plan* split, const int64_t* u_off, const int64_t* vt_off, const int64_t* keep,
                            const double* S_host, const int64_t* s_off, int32_t l2r, qcm_plan** plan);

/* The product of a site tensor with a block-diagonal bond factor N, the second
 * half of mergeUnitaryFactor (SweepBasedAlgorithms/SweepMPSUpdater.h:237-250):
 * from_left != 0: MPSTensor::multiply_from_left (mp_tensors/mpstensor.hpp:
 * 314-321): N . T over T's left bond (T made right-paired, N's left basis the new
 * left index, the result back to left-paired); from_left = 0: multiply_from_right
 * (:302-309): T . N over the right bond.  Blocks multiply where N's right charge
 * (from_left) or left charge meets T's.  Slots: KET = T (left-paired), LEFT = N;
 * OUT = the new tensor, left-paired (layout and indices through
 * qcm_plan_out_tensor).  FP64 grouped products and gather maps. */
int qcm_plan_mps_multiply(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                          const qcm_blocks_t* t, const qcm_blocks_t* n, int32_t from_left, qcm_plan** plan);

/* A site tensor between its pairings (reshape_left_to_right / reshape_right_to_left,
 * mp_tensors/reshapes.h): to_right != 0: KET left-paired -> OUT right-paired;
 * else KET right-paired -> OUT left-paired.  The indices are unchanged; the output
 * blocks through qcm_plan_out_tensor. */
int qcm_plan_mps_reshape(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                         const qcm_blocks_t* t, int32_t to_right, qcm_plan** plan);

/* Charge-matched product of two block matrices, OUT = op(A) op(B) with op the
 * transpose where ta / tb != 0 (block_matrix gemm and transpose,
 * dmrg/framework/dmrg/block_matrix/block_matrix_algorithms.h:47-80, :118-128):
 * every pair of blocks whose inner charges agree adds its product to the output
 * block (left charge of op(A), right charge of op(B)).  A in slot KET, B in slot
 * LEFT; output blocks through qcm_plan_out_tensor (indices empty).  FP64; run
 * with qcm_plan_run / qcm_ctx_run.  Used for the products of the density-matrix
 * truncation: U^T theta, theta U. */
int qcm_plan_block_gemm(const qcm_blocks_t* a, int32_t ta, const qcm_blocks_t* b, int32_t tb, qcm_plan** plan);

/* Density matrix of the heev truncation (TwoSiteTensor::predict_split_l2r/r2l,
 * dmrg/framework/dmrg/mp_tensors/twositetensor.hpp:184-297; predict_new_state_*,
 * mp_tensors/contractions/common/prediction.hpp:19-125): OUT = theta theta^T (l2r,
 * theta left-paired) or theta^T theta (r2l, theta right-paired), theta in slot KET;
 * with alpha != 0 and half != NULL, plus alpha sum_b h_b h_b^T (l2r) or
 * alpha sum_b h_b^T h_b (r2l) over the boundary tensor product h in slot RIGHT
 * (qcm_plan_boundary_tensor_mpo's output): per bond b, every pair of h[b]'s blocks
 * sharing their right (l2r) / left (r2l) charge whose output charges (ci, cj) are
 * a block of theta.  Output blocks through qcm_plan_out_tensor.  FP64. */
int qcm_plan_density_matrix(const qcm_blocks_t* theta, int32_t l2r, const qcm_boundary_t* half, double alpha,
                            qcm_plan** plan);

/* Output tensor of an MPS-level plan: block list (q: 4 per block, rows, cols,
 * element offsets) and its three indices (physical, left, right) concatenated:
 * n_idx3[i] sectors each, charges idx_q (2 per sector) and sizes idx_size.
 * Call with NULL arrays first for the counts. */
int qcm_plan_out_tensor(const qcm_plan* plan, int32_t which, int32_t* nblocks, int32_t* q, int64_t* rows,
                        int64_t* cols, int64_t* off, int32_t* n_idx3, int32_t* idx_q, int64_t* idx_size);

/* ---------------------------------------------------------------- factorisations
 * Batched FP64 SVD of independent column-major blocks by one-sided Jacobi, on
 * the GPU: replaces the per-block LAPACK calls of the truncation and
 * canonicalisation steps -- gesvd in svd_truncate (dmrg/framework/dmrg/
 * block_matrix/block_matrix_algorithms.h:163-333), heevd in heev_truncate
 * (:387-440; for a symmetric positive semi-definite block the SVD is its
 * eigendecomposition, eigenvalues descending), and the QR / LQ of
 * leftNormalizeAndReturn / rightNormalizeAndReturn (:442-492, mp_tensors/
 * mpstensor.hpp:219-258; U and S.Vt serve as the orthonormal factor and the
 * remainder).  Block k is rows[k] x cols[k] at element src_off[k] of the
 * source (ld = rows); it yields k_k = min(rows, cols) singular values,
 * descending, U (rows x k_k, ld rows) and Vt (k_k x cols, ld k_k), packed
 * block after block (qcm_svd_block_offsets).  The workspace holds the
 * rotated block and the accumulated rotations (qcm_svd_sizes).  Rounds run
 * until no pair of columns is rotated in a whole sweep (|a.b| <= sqrt(p) eps |a||b|,
 * p = max(rows, cols), the threshold of LAPACK's one-sided Jacobi);
 * a block still rotating after 40 sweeps makes qcm_svd_run return
 * QCM_E_RANGE.  min(rows, cols) <= 4096 per block.  A round pairs panels of
 * bw columns, each pair rotated in shared memory (bw = 16 or 8, the widest whose
 * panels of W and V fit for the tallest block; qcm_svd_panel_width), or single
 * columns (bw = 0) when neither fits; qcm_svd_set_panel_width picks another width
 * (0, 2, 4, 8, 16) before the first run (the same factorisation up to rounding). */
typedef struct qcm_svd qcm_svd;
int qcm_svd_create(int32_t nblocks, const int64_t* rows, const int64_t* cols, const int64_t* src_off, qcm_svd** out);
int qcm_svd_sizes(const qcm_svd* svd, int64_t* work_elems, int64_t* u_elems, int64_t* s_elems, int64_t* vt_elems);
int qcm_svd_block_offsets(const qcm_svd* svd, int64_t* s_off, int64_t* u_off, int64_t* vt_off);
int qcm_svd_run(qcm_svd* svd, const double* src, double* work, double* U, double* S, double* Vt, void* stream);
/* Sweeps of the widest block in the last run (host polls once per such sweep). */
int qcm_svd_last_sweeps(const qcm_svd* svd, int32_t* sweeps);
int qcm_svd_set_panel_width(qcm_svd* svd, int32_t bw);
int qcm_svd_panel_width(const qcm_svd* svd, int32_t* bw);
void qcm_svd_destroy(qcm_svd* svd);


/* The global cut of estimate_truncation on the device: vals_dev holds each
 * block's values in descending order, block k at [blk_off[k], blk_off[k+1])
 * (host array).  evalscut = max(cutoff * s0, s[Mmax]); every value >= evalscut
 * is kept (Mmax + 1 values when there is no tie, as the reference keeps them);
 * keep[k] (host) = values kept of block k.  mode 0: singular values, weight =
 * discarded sum of s^2 / sum of s^2; mode 1: density-matrix eigenvalues, both
 * weight fields = the discarded fraction (as heev_truncate reports them).  At
 * most 16384 values.  Synchronises the stream. */
int qcm_truncation_cut(const double* vals_dev, int32_t nblocks, const int64_t* blk_off, int64_t Mmax, double cutoff,
                       int32_t mode, int64_t* keep, qcm_trunc_t* out, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QCM_GB300_H */
