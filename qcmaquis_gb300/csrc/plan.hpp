// Internal data structures of the contraction plans.
//
// A plan is a list of stages.  Each stage is one of
//   ZERO  : clear a range of a buffer,
//   AXPY  : gather-accumulate tiles  D = sum_t alpha_t * S_t   (overwrite),
//   GEMM  : grouped block products   C = sum_s alpha_s * op(A_s) op(B_s) (overwrite).
// Every output tile is owned by exactly one work item, so results do not
// depend on scheduling (the reference accumulates under an OpenMP critical
// section, ct/non-abelian/site_hamil.hpp:141-143, whose order varies).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <utility>
#include <vector>

#include "qcm_gb300.h"

namespace qcm {

struct Q {
    int n = 0, s = 0;  // (N, 2S)
    Q() = default;
    Q(int n_, int s_) : n(n_), s(s_) {}
    bool operator<(const Q& o) const { return n < o.n || (n == o.n && s < o.s); }
    bool operator>(const Q& o) const { return o < *this; }
    bool operator==(const Q& o) const { return n == o.n && s == o.s; }
    bool operator!=(const Q& o) const { return !(*this == o); }
};
inline Q fuse(Q a, Q b) { return Q(a.n + b.n, a.s + b.s); }

// QCM_SYM_* of a tensor or plan: true for the abelian groups (TwoU1, U1), which
// share the abelian contraction rules; throws on a code that names no group.
bool abelian_symmetry(int32_t symmetry);
inline Q neg(Q a) { return Q(-a.n, -a.s); }
inline bool triangle(int a, int b, int c) { return ((a + b + c) % 2 == 0) && std::abs(a - b) <= c && c <= a + b; }

// Sorted-descending quantum-number index.
struct Idx {
    std::vector<std::pair<Q, int64_t>> d;
    size_t size() const { return d.size(); }
    size_t position(Q c) const;
    bool has(Q c) const { return position(c) < d.size(); }
    int64_t size_of(Q c) const;
    void insert(Q c, int64_t s);
    void sort();
};
Idx index_product(const Idx& a, const Idx& b);
Idx adjoin(const Idx& a);
void common_subset(Idx& a, Idx& b);

struct PB {
    std::map<std::pair<Q, Q>, int64_t> keys;
    std::map<Q, int64_t> sizes;
    PB(const Idx& a, const Idx& b, bool neg_first);
    int64_t operator()(Q a, Q b) const;
    int64_t size(Q c) const;
};

struct Blk {
    Q lc, rc;
    int64_t rows = 0, cols = 0, off = 0;
    int64_t ld = 0;   // leading dimension when padded (0: rows)
    int64_t pitch() const { return ld ? ld : rows; }
};

// Block list in DualIndex order (descending on (lc, rc)).
struct BM {
    std::vector<Blk> b;
    size_t find(Q lc, Q rc) const;
    size_t left_lower_bound(Q lc) const;
    size_t insert(Blk x);  // returns position
    int64_t assign_offsets(int64_t base);  // sequential offsets, returns end
    // offsets rounded up to multiples of align elements and, for blocks of at least
    // 32 rows, leading dimensions too (16-byte aligned columns for align = 4 FP32
    // elements); returns end
    int64_t assign_offsets_aligned(int64_t base, int64_t align);
};

// Allocator that default-initialises (no zero fill when a table of PODs is resized
// before every element is written in parallel).
template <class T>
struct DefaultInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = DefaultInitAlloc<U>; };
    DefaultInitAlloc() = default;
    template <class U> DefaultInitAlloc(const DefaultInitAlloc<U>&) noexcept {}
    template <class U> void construct(U* p) noexcept { ::new ((void*)p) U; }
    template <class U, class... A> void construct(U* p, A&&... a) { ::new ((void*)p) U(std::forward<A>(a)...); }
};

struct AxpyOut {
    int32_t dst_buf;
    int64_t dst_off, ldd, rows, cols;
    int64_t t_begin, t_end;
};
struct AxpyTerm {
    int32_t src_buf;
    int64_t src_off, lds;
    double alpha;
};
struct GemmOut {
    int32_t c_buf;
    int64_t c_off, ldc, M, N;
    int64_t s_begin, s_end;
    // 1: the output's columns are 16-byte aligned and padded to a multiple of 4
    // rows that nothing reads into a result (the K1 result T), so a store may
    // write whole groups of 4 rows
    int32_t vec_store = 0;
};
struct GemmSeg {
    int32_t a_buf, ta;
    int64_t a_off, lda;
    int32_t b_buf, tb;
    int64_t b_off, ldb;
    int64_t K;
    double alpha;
};

// ST_DOT: the adjoint of a gather-axpy stage -- for every term k of the axpy
// tables (aout/aterm), g[k] = <source tile, output-adjoint tile>, written to
// dot_buf; then OUT[tt] = sum over the terms of parameter tt of dot_w[k] g[k]
enum StageKind { ST_AXPY = 0, ST_GEMM = 1, ST_ZERO = 2, ST_DOT = 3 };

// ---- operand images of the BF16x3 tensor-core executor
// An image holds one operand panel (R rows x K, K-major as the MMA reads it)
// split into three BF16 slices, in the shared-memory order of the UMMA
// canonical K-major no-swizzle layout: for K-chunk c (32 elements, 64 bytes
// per row) and slice s, 8-row group g occupies 512 bytes at
// img_off + ((c*3 + s)*G + g)*512; inside it, core matrix q (8 K-elements)
// at q*128, row r%8 at 16-byte steps.  Rows are padded to G*8, K to the chunk
// size, with zeros.
struct ImgPanel {
    int64_t src_off;   // element offset of the source block (kcontig 2: offset into the gather table)
    int64_t img_off;   // byte offset of the image in the image buffer (multiple of 512)
    int32_t src_buf, ld, R, K, kcontig, G;
    // kcontig 0: element (r,k) at src_off + r + k*ld; 1: at src_off + r*ld + k;
    // 2: at gather[src_off + k] + r (column k is a contiguous source tile)
};
// One output of the image executor, tile element (i, j) with i along the MMA
// M side and j along N: mode 0 writes c_off + i*si + j*sj; mode 1 writes
// off_j + (i % rows) + (i / rows)*ld_j with (off_j, ld_j) = coltab pair
// ctab + j (column j is one output tile).
struct ImgOut {
    int64_t c_off, si, sj, ctab;
    int32_t c_buf, mrows, ncols, mode, rows, pad;
};
// ImgSeg.flags: IMG_B_CONST -- the B image lives in the plan's constant images.
enum { IMG_B_CONST = 2 };
struct ImgSeg {
    int64_t a_img, b_img;   // byte offsets of the A and B panel images (at the chunk range start)
    int32_t a_G, b_G, kc;   // row groups of the panels, K-chunks
    float alpha;
    int32_t flags, a_panel, a_c0, pad;   // a_panel / a_c0: the A panel and its first chunk (inspection)
};
struct ImgUnit {
    int32_t out, m0, n0, nt, s_begin, s_end;  // nt: MMA N (multiple of 16, <= 128)
};
struct ImgTables {
    std::vector<ImgPanel> panels;
    std::vector<int32_t> build;   // (panel, chunk) pairs, one image-builder CTA each
    std::vector<ImgOut> outs;
    std::vector<ImgSeg> segs;
    std::vector<ImgUnit> units;
    std::vector<int64_t> gather;  // source offsets of gathered panels (kcontig 2)
    std::vector<int64_t> coltab;  // (offset, ld) pairs of the output tiles of mode-1 outputs
    std::vector<uint8_t, DefaultInitAlloc<uint8_t>> cimg;  // constant images (coefficient matrices), built by the plan
    int64_t bytes = 0;            // per-call image bytes
    // A-resident mode: every tile is one segment of at most IMG_ARES_MAX K-chunks,
    // tiles are ordered by their A tile (image, m0), and each CTA takes a
    // contiguous cost-balanced range of them, so that a run of tiles sharing one
    // A tile loads it into shared memory once and streams only B.
    bool ares = false;
    std::vector<int64_t> cost;    // prefix sums of the tile costs (size tiles + 1)
};
constexpr int IMG_ARES_MAX = 5;
// n_tile_max: widest N of a tile (16..128, multiple of 16); a_resident: the K1 A-resident
// schedule when every tile is one short block product
void build_image_tables(const struct Stage& st, ImgTables& t, int n_tile_max = 128, bool a_resident = false);
// Dense groups of a gather-axpy stage: output tiles that share their sources
// (a connected component of the output/source graph), have at least
// min_terms terms and one tile shape become one block product
// contr[:, group] = T_gathered . W^T on the tensor cores.  heavy[o] marks the
// outputs taken.
void build_dense_groups(const struct Stage& st, int64_t min_terms, ImgTables& t, std::vector<char>& heavy);
// Connected components of a gather-axpy stage's output/source graph (outputs
// that share a source tile, transitively): root[i] = smallest output of i's
// component.  Returns false when some term's source is not a contiguous tile.
bool axpy_components(const struct Stage& st, std::vector<int32_t>& root);
// The pitch of a gather output tile whose sources share one leading dimension
// between rows and rows rounded up to 4 (the padded K1 result): the tile is then
// a contiguous pitch x cols run of each source; -1 for other strided sources.
int64_t tile_pitch(const struct Stage& st, const AxpyOut& a);

struct Stage {
    int kind;
    // ZERO
    int32_t zbuf = 0;
    int64_t zoff = 0, zlen = 0;
    // AXPY
    std::vector<AxpyOut, DefaultInitAlloc<AxpyOut>> aout;
    std::vector<AxpyTerm, DefaultInitAlloc<AxpyTerm>> aterm;
    // GEMM
    std::vector<GemmOut> gout;
    std::vector<GemmSeg> gseg;
    // device copies (owned)
    void* d_a = nullptr;
    void* d_b = nullptr;
    void* d_c = nullptr;  // work list (FP64 executor, 64 x 64 tiles)
    int64_t n_work = 0;
    void* d_tcw = nullptr;  // work list (tensor-core executor, 128 x 64 tiles)
    int64_t n_tcw = 0;
    int32_t src_buf = -1;   // AXPY: the one buffer all terms read (-2: several)
    void* d_cw = nullptr;   // AXPY: chunk work list of the contiguous-source executor
    int64_t n_cw = 0;       // 0: some term's source is not contiguous (generic executor)
    // GEMM: tables of the BF16x3 image executor; AXPY: its dense groups
    ImgTables img;
    std::vector<char> heavy;     // AXPY: outputs computed by the dense groups
    std::vector<int32_t> comp_root;  // AXPY: connected components (axpy_components), when computed
    void* d_igather = nullptr;
    void* d_icoltab = nullptr;
    void* d_icimg = nullptr;
    void* d_cw_light = nullptr;  // AXPY: chunk work list of the outputs outside the dense groups
    int64_t n_cw_light = 0;
    // AXPY with dense groups: side stream and fork/join events, so that the gather of
    // the other outputs runs alongside the dense groups' block products
    void* side_stream = nullptr;
    void* ev_fork = nullptr;
    void* ev_join = nullptr;
    void* d_ipanel = nullptr;
    void* d_ibuild = nullptr;
    void* d_iout = nullptr;
    void* d_iseg = nullptr;
    void* d_iunit = nullptr;
    void* d_icost = nullptr;
    // DOT: per-term weight and parameter index, the buffer of the per-term dots,
    // the number of parameters; device: terms, parameter-sorted term lists, weights
    std::vector<double> dot_w;
    std::vector<int32_t> dot_tt;
    int32_t dot_buf = 0;
    int32_t n_tt = 0;
    void* d_dterm = nullptr;
    void* d_dptr = nullptr;
    void* d_didx = nullptr;
    void* d_dw = nullptr;
};

// PK_GRAD: gradient of <psi| H_eff |psi> with respect to every MPO term scale
// PK_DIAG: the diagonal of H_eff (FP64 only)
// PK_THETA: two-site tensor from two site tensors; PK_SPLIT: both-paired two-site
// tensor from the reduced one; PK_ASSEMBLE: the site tensors of a truncated split;
// PK_MPS: one site tensor from another (a reshape, or the product with a factor)
enum PlanKind { PK_SIGMA = 0, PK_BLEFT = 1, PK_BRIGHT = 2, PK_GRAD = 3, PK_DIAG = 4, PK_THETA = 5, PK_SPLIT = 6,
                PK_ASSEMBLE = 7, PK_MPS = 8 };

}  // namespace qcm

struct qcm_plan {
    int kind;
    std::vector<qcm::Stage> stages;
    int64_t out_elems = 0;
    int64_t scratch[3] = {0, 0, 0};
    int64_t image_bytes = 0;  // image buffer of the BF16x3 image executor
    int32_t last_kernels = 0; // kernels the last run launched (memsets excluded)
    // output boundary layout (boundary plans)
    std::vector<int32_t> out_blk_ptr;
    std::vector<qcm::Blk> out_blocks;
    double gemm_flops = 0, axpy_flops = 0, axpy_bytes = 0;
    // output tensor of an MPS-level plan (PK_THETA / PK_SPLIT / PK_ASSEMBLE): its block
    // layout and its indices (physical, left, right); PK_ASSEMBLE has a second output
    // (the right site, slot OUT2 = S2) in out2_*
    std::vector<qcm::Blk> out_bm;
    qcm::Idx out_phys, out_left, out_right;
    std::vector<qcm::Blk> out2_bm;
    qcm::Idx out2_phys, out2_left, out2_right;
    bool uploaded = false;
    int device = -1;
    // (stream, event recorded on it after the plan's last run there): the teardown
    // frees the tables once every stream has passed its event
    std::vector<std::pair<void*, void*>> run_ev;
    bool captured = false;  // ran inside a stream capture: the teardown waits for the device
};

namespace qcm {
void set_error(const std::string& msg);
Idx read_index(const qcm_index_t* x);
BM read_blocks(const qcm_blocks_t* x);
std::vector<BM> read_boundary(const qcm_boundary_t* x);
qcm_plan* build_block_gemm(const BM& a, bool ta, const BM& b, bool tb);
qcm_plan* build_density_matrix(const BM& theta, bool l2r, const std::vector<BM>* half, double alpha);
qcm_plan* build_split(const Idx& p1, const Idx& p2, const Idx& left_i, const Idx& right_i, const BM& u,
                      bool abelian);
qcm_plan* build_assemble(const Idx& p1, const Idx& p2, const Idx& left_i, const Idx& right_i, const BM& both,
                         const int64_t* u_off, const int64_t* vt_off, const int64_t* kdim, const int64_t* keep,
                         const double* S_host, const int64_t* s_off, bool l2r);
double wigner6j(int, int, int, int, int, int);
double wigner9j(int, int, int, int, int, int, int, int, int);
void set_coupling(int a, int b, int c, int d, int e, int f, int g, int h, int i, double init, double out[4]);
double conjugate_correction(int lc_spin, int rc_spin, int tensor_spin);
// releases a plan's device tables (stream-ordered after its runs; see qcm_plan_destroy)
void release_plan_device(struct ::qcm_plan* p);
int tc_build_work(const Stage& st, std::vector<int64_t>& w);
int tc_img_launch(const Stage& st, double* const* bufs, uint32_t f32mask, void* stream, int nprod = 6);
int tc_launch(const void* d_out, const void* d_seg, const void* d_work, int64_t n_work, double* const* bufs,
              uint32_t f32mask, int precision, void* stream);
}  // namespace qcm
