// Contraction-plan builder: quantum-number block pairing and index maps for the
// SU2U1 sigma vector and boundary updates, emitted as deterministic task lists.
//
// The traversals restate, block for block:
//   BoundaryMPSProduct / MPSBoundaryProduct  ct/common/boundary_times_mps.hpp:163-385
//   SU2::gemm_trim_left / gemm_trim_right / gemm_trim / gemm
//                                            ct/non-abelian/gemm.hpp:48-204
//   SU2::lbtm_kernel + detail::lbtm          ct/non-abelian/apply_op.hpp:23-101,
//                                            ct/non-abelian/micro_kernels.hpp:19-45
//   SU2::rbtm_tasks + rbtm_axpy + task_axpy  ct/non-abelian/apply_op.hpp:114-232,
//                                            ct/non-abelian/micro_kernels.hpp:143-198
//   site_hamil_lbtm                          ct/non-abelian/site_hamil.hpp:57-147
//   overlap_mpo_left_step / _right_step      ct/common/move_boundary.hpp:128-229
//   reshape_left_to_right_new                mp_tensors/reshapes.h:178-221
// but instead of performing each axpy/GEMM immediately they record it, grouped
// by the output tile it writes, so the device executes every output exactly
// once without atomics.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <numeric>
#include <stdexcept>
#include <thread>
#include <tuple>
#include <unordered_map>

#include "plan.hpp"

namespace qcm {

bool abelian_symmetry(int32_t symmetry) {
    if (symmetry == QCM_SYM_SU2U1) return false;
    if (symmetry == QCM_SYM_TWOU1 || symmetry == QCM_SYM_U1) return true;
    throw std::runtime_error("unknown symmetry " + std::to_string(symmetry));
}

// f(0) .. f(n - 1) on up to 16 host threads, tasks taken in order from a shared
// counter; the first exception a task throws is rethrown here
static void parallel_for(size_t n, const std::function<void(size_t)>& f) {
    std::atomic<size_t> next{0};
    std::mutex err_mu;
    std::string err;
    auto worker = [&]() {
        for (;;) {
            const size_t i = next.fetch_add(1);
            if (i >= n) return;
            try {
                f(i);
            } catch (const std::exception& ex) {
                std::lock_guard<std::mutex> g(err_mu);
                if (err.empty()) err = ex.what();
            }
        }
    };
    const unsigned nt = (unsigned)std::min<size_t>(n, std::max(1u, std::min(16u, std::thread::hardware_concurrency())));
    std::vector<std::thread> pool;
    for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
    worker();
    for (auto& th : pool) th.join();
    if (!err.empty()) throw std::runtime_error(err);
}

// A-resident mode for single-segment stages (K1).  Off: measured slower at the
// benchmark size, because contiguous per-CTA tile ranges lose the L2 reuse of
// the B operand across CTAs that the strided order has.
static constexpr bool kAResident = false;   // default of the K1 schedule option
// column alignment (elements) of the K1 result T in the sigma and boundary plans
// (16 bytes in FP32: vector stores in the image epilogue)
static constexpr int64_t kTAlign = 4;

static thread_local std::string g_err;
void set_error(const std::string& msg) { g_err = msg; }

// ------------------------------------------------------------------ indices
size_t Idx::position(Q c) const {
    // descending order: binary search
    size_t lo = 0, hi = d.size();
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (d[mid].first > c) lo = mid + 1; else hi = mid;
    }
    if (lo < d.size() && d[lo].first == c) return lo;
    return d.size();
}
int64_t Idx::size_of(Q c) const {
    size_t p = position(c);
    if (p == d.size()) throw std::runtime_error("charge not in index");
    return d[p].second;
}
void Idx::insert(Q c, int64_t s) {
    size_t pos = 0;
    while (pos < d.size() && !(d[pos].first < c)) ++pos;
    d.insert(d.begin() + pos, {c, s});
}
void Idx::sort() {
    std::stable_sort(d.begin(), d.end(), [](const std::pair<Q, int64_t>& a, const std::pair<Q, int64_t>& b) {
        return a.first > b.first;
    });
}
Idx index_product(const Idx& a, const Idx& b) {
    std::map<Q, int64_t> acc;
    for (auto& x : a.d)
        for (auto& y : b.d) acc[fuse(x.first, y.first)] += x.second * y.second;
    Idx r;
    for (auto it = acc.rbegin(); it != acc.rend(); ++it) r.d.push_back({it->first, it->second});
    return r;
}
Idx adjoin(const Idx& a) {
    Idx r;
    for (auto& x : a.d) r.d.push_back({neg(x.first), x.second});
    r.sort();
    return r;
}
void common_subset(Idx& a, Idx& b) {
    Idx na, nb;
    for (auto& x : a.d)
        if (b.has(x.first)) na.d.push_back(x);
    for (auto& x : b.d)
        if (na.has(x.first)) nb.d.push_back(x);
    a = na;
    b = nb;
}
PB::PB(const Idx& a, const Idx& b, bool neg_first) {
    for (auto& x : a.d)
        for (auto& y : b.d) {
            Q pc = neg_first ? fuse(neg(x.first), y.first) : fuse(x.first, y.first);
            int64_t cur = sizes.count(pc) ? sizes[pc] : 0;
            keys[{x.first, y.first}] = cur;
            sizes[pc] = cur + x.second * y.second;
        }
}
int64_t PB::operator()(Q a, Q b) const {
    auto it = keys.find({a, b});
    if (it == keys.end()) throw std::runtime_error("product basis key missing");
    return it->second;
}
int64_t PB::size(Q c) const {
    auto it = sizes.find(c);
    if (it == sizes.end()) throw std::runtime_error("product basis sector missing");
    return it->second;
}

static bool key_gt(const Blk& a, Q lc, Q rc) { return a.lc > lc || (a.lc == lc && a.rc > rc); }

size_t BM::find(Q lc, Q rc) const {
    size_t lo = 0, hi = b.size();
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (key_gt(b[mid], lc, rc)) lo = mid + 1; else hi = mid;
    }
    if (lo < b.size() && b[lo].lc == lc && b[lo].rc == rc) return lo;
    return b.size();
}
size_t BM::left_lower_bound(Q lc) const {
    size_t lo = 0, hi = b.size();
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (b[mid].lc > lc) lo = mid + 1; else hi = mid;
    }
    return lo;
}
size_t BM::insert(Blk x) {
    size_t lo = 0, hi = b.size();
    while (lo < hi) {
        size_t mid = (lo + hi) / 2;
        if (key_gt(b[mid], x.lc, x.rc)) lo = mid + 1; else hi = mid;
    }
    b.insert(b.begin() + lo, x);
    return lo;
}
static void check_block_extent(const Blk& x) {
    // the executors use 32-bit in-block offsets
    if (x.rows * x.cols >= (int64_t(1) << 31) || x.rows >= (int64_t(1) << 31) || x.cols >= (int64_t(1) << 31))
        throw std::runtime_error("block larger than 2^31 elements");
}

int64_t BM::assign_offsets(int64_t base) {
    for (auto& x : b) {
        check_block_extent(x);
        x.off = base;
        base += x.rows * x.cols;
    }
    return base;
}

int64_t BM::assign_offsets_aligned(int64_t base, int64_t align) {
    if (align <= 1) return assign_offsets(base);
    for (auto& x : b) {
        check_block_extent(x);
        // columns of fewer than 32 rows stay unpadded: their padding would be a large
        // share of the tile, and the gather's short tiles read contiguous runs anyway
        x.ld = x.rows < 32 ? x.rows : (x.rows + align - 1) / align * align;
        x.off = (base + align - 1) / align * align;
        base = x.off + x.ld * x.cols;
    }
    return base;
}

// ------------------------------------------------------------------ Wigner symbols (Racah)
static long double lfact(int n) {
    static std::vector<long double> t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.resize(400);
        t[0] = 1.0L;
        for (int i = 1; i < 400; ++i) t[i] = t[i - 1] * (long double)i;
    });
    if (n < 0 || n >= 400) throw std::runtime_error("factorial argument out of range");
    return t[n];
}
static long double delta2(int a, int b, int c) {
    return lfact((a + b - c) / 2) * lfact((a - b + c) / 2) * lfact((-a + b + c) / 2) / lfact((a + b + c) / 2 + 1);
}
static long double sixj_ld(int j1, int j2, int j3, int j4, int j5, int j6) {
    if (!(triangle(j1, j2, j3) && triangle(j1, j5, j6) && triangle(j4, j2, j6) && triangle(j4, j5, j3))) return 0.0L;
    int a1 = (j1 + j2 + j3) / 2, a2 = (j1 + j5 + j6) / 2, a3 = (j4 + j2 + j6) / 2, a4 = (j4 + j5 + j3) / 2;
    int b1 = (j1 + j2 + j4 + j5) / 2, b2 = (j2 + j3 + j5 + j6) / 2, b3 = (j3 + j1 + j6 + j4) / 2;
    int tmin = std::max(std::max(a1, a2), std::max(a3, a4)), tmax = std::min(b1, std::min(b2, b3));
    long double s = 0.0L;
    for (int t = tmin; t <= tmax; ++t) {
        long double term = lfact(t + 1) / (lfact(t - a1) * lfact(t - a2) * lfact(t - a3) * lfact(t - a4) *
                                           lfact(b1 - t) * lfact(b2 - t) * lfact(b3 - t));
        s += (t % 2) ? -term : term;
    }
    long double pref = delta2(j1, j2, j3) * delta2(j1, j5, j6) * delta2(j4, j2, j6) * delta2(j4, j5, j3);
    return s * sqrtl(pref);
}
double wigner6j(int a, int b, int c, int d, int e, int f) { return (double)sixj_ld(a, b, c, d, e, f); }
double wigner9j(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    if (!(triangle(a, b, c) && triangle(d, e, f) && triangle(g, h, i) && triangle(a, d, g) && triangle(b, e, h) &&
          triangle(c, f, i)))
        return 0.0;
    int xmin = std::max(std::abs(a - i), std::max(std::abs(h - d), std::abs(b - f)));
    int xmax = std::min(a + i, std::min(h + d, b + f));
    long double tot = 0.0L;
    for (int x = xmin; x <= xmax; x += 2) {
        long double t = sixj_ld(a, d, g, h, i, x) * sixj_ld(b, e, h, d, x, f) * sixj_ld(c, f, i, x, a, b);
        t *= (long double)(x + 1);
        tot += (x % 2) ? -t : t;
    }
    return (double)tot;
}
static double mod_coupling(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    return std::sqrt((g + 1.0) * (h + 1.0) * (c + 1.0) * (f + 1.0)) * wigner9j(a, b, c, d, e, f, g, h, i);
}
// set_coupling(..., init) = init * F(a..i); F depends only on the nine doubled
// spins (all small), so it is cached per thread.
struct CouplingVal { double v[4]; };
static void coupling_unit(int a, int b, int c, int d, int e, int f, int g, int h, int i, double out[4]);

void set_coupling(int a, int b, int c, int d, int e, int f, int g, int h, int i, double init, double out[4]) {
    static thread_local std::unordered_map<uint64_t, CouplingVal> cache;
    const int args[9] = {a, b, c, d, e, f, g, h, i};
    uint64_t key = 0;
    bool packable = true;
    for (int x : args) {
        if (x < 0 || x >= 128) { packable = false; break; }
        key = (key << 7) | (uint64_t)x;
    }
    if (packable) {
        auto it = cache.find(key);
        if (it == cache.end()) {
            CouplingVal cv;
            coupling_unit(a, b, c, d, e, f, g, h, i, cv.v);
            it = cache.emplace(key, cv).first;
        }
        for (int k = 0; k < 4; ++k) out[k] = init * it->second.v[k];
        return;
    }
    coupling_unit(a, b, c, d, e, f, g, h, i, out);
    for (int k = 0; k < 4; ++k) out[k] *= init;
}

static void coupling_unit(int a, int b, int c, int d, int e, int f, int g, int h, int i, double out[4]) {
    double pref = std::sqrt((i + 1.0) * (a + 1.0) / ((g + 1.0) * (c + 1.0)));
    out[0] = out[1] = out[2] = out[3] = 0.0;
    if (triangle(a, b, c)) {
        out[0] = pref * mod_coupling(a, b, c, d, e, f, g, h, i);
        out[2] = pref * mod_coupling(a, b, c, d, e, f, g, 2, i);
    }
    if (triangle(a, 2, c)) {
        out[1] = pref * mod_coupling(a, 2, c, d, e, f, g, h, i);
        out[3] = pref * mod_coupling(a, 2, c, d, e, f, g, 2, i);
    }
}
double conjugate_correction(int lc, int rc, int S) {
    int Sm = std::min(rc, lc), diff = rc - lc;
    if (S == 0) return 1.0;
    if (S == 1) {
        if (diff > 0) return -std::sqrt((Sm + 1.0) / (Sm + 2.0));
        if (diff < 0) return std::sqrt((Sm + 2.0) / (Sm + 1.0));
        return 0.0;
    }
    if (S == 2) {
        if (diff > 0) return -std::sqrt((Sm + 1.0) / (Sm + 3.0));
        if (diff < 0) return -std::sqrt((Sm + 3.0) / (Sm + 1.0));
        return 1.0;
    }
    throw std::runtime_error("hermitian conjugate for reduced tensor operators only implemented up to rank 1");
}

// ------------------------------------------------------------------ views of the C-ABI inputs
Idx read_index(const qcm_index_t* x) {
    Idx r;
    if (!x) throw std::runtime_error("null index");
    for (int i = 0; i < x->n; ++i) r.d.push_back({Q(x->q[2 * i], x->q[2 * i + 1]), x->size[i]});
    for (size_t i = 1; i < r.d.size(); ++i)
        if (!(r.d[i - 1].first > r.d[i].first)) throw std::runtime_error("index not sorted descending");
    return r;
}
BM read_blocks(const qcm_blocks_t* x) {
    BM r;
    if (!x) throw std::runtime_error("null block list");
    for (int k = 0; k < x->n; ++k) {
        Blk b;
        b.lc = Q(x->q[4 * k], x->q[4 * k + 1]);
        b.rc = Q(x->q[4 * k + 2], x->q[4 * k + 3]);
        b.rows = x->rows[k];
        b.cols = x->cols[k];
        b.off = x->off[k];
        if (b.rows < 0 || b.cols < 0 || b.off < 0) throw std::runtime_error("negative block extent");
        check_block_extent(b);
        if (!r.b.empty() && !key_gt(r.b.back(), b.lc, b.rc)) throw std::runtime_error("blocks not in DualIndex order");
        r.b.push_back(b);
    }
    return r;
}
std::vector<BM> read_boundary(const qcm_boundary_t* x) {
    if (!x) throw std::runtime_error("null boundary");
    std::vector<BM> r(x->aux);
    for (int b = 0; b < x->aux; ++b) {
        for (int k = x->blk_ptr[b]; k < x->blk_ptr[b + 1]; ++k) {
            Blk bl;
            bl.lc = Q(x->q[4 * k], x->q[4 * k + 1]);
            bl.rc = Q(x->q[4 * k + 2], x->q[4 * k + 3]);
            bl.rows = x->rows[k];
            bl.cols = x->cols[k];
            bl.off = x->off[k];
            if (bl.rows < 0 || bl.cols < 0 || bl.off < 0) throw std::runtime_error("negative block extent");
            check_block_extent(bl);
            if (!r[b].b.empty() && !key_gt(r[b].b.back(), bl.lc, bl.rc))
                throw std::runtime_error("boundary blocks not in DualIndex order");
            r[b].b.push_back(bl);
        }
    }
    return r;
}

struct MpoV {
    const qcm_mpo_t* m;
    std::vector<std::vector<int>> row_b2;        // b1 -> sorted b2
    std::vector<std::vector<int>> row_elem;      // b1 -> element ids (matching row_b2)
    MpoV(const qcm_mpo_t* m_) : m(m_) {
        if (!m) throw std::runtime_error("null mpo");
        abelian_symmetry(m->symmetry);
        row_b2.resize(m->row_dim);
        row_elem.resize(m->row_dim);
        for (int b2 = 0; b2 < m->col_dim; ++b2)
            for (int e = m->col_ptr[b2]; e < m->col_ptr[b2 + 1]; ++e) {
                int b1 = m->row_of[e];
                if (b1 < 0 || b1 >= m->row_dim) throw std::runtime_error("mpo row index out of range");
                row_b2[b1].push_back(b2);
                row_elem[b1].push_back(e);
            }
        for (int o = 0; o < m->n_ops; ++o)
            for (int k = m->op_blk_ptr[o]; k < m->op_blk_ptr[o + 1]; ++k)
                if (m->blk_ent_ptr[k] > m->blk_ent_ptr[k + 1]) throw std::runtime_error("bad op entries");
    }
    int lspin(int b) const { return m->left_spin[b]; }
    int rspin(int b) const { return m->right_spin[b]; }
    // Abelian groups (TwoU1, U1) have no spin couplings: every coupling is the term's
    // scale, every triangle test passes and a Hermitian partner enters with
    // scale 1 (conjugate_phases of common/boundary_times_mps.hpp:44-51 and the
    // abelian lbtm/rbtm kernels, ct/abelian/apply_op.hpp:80-138).
    bool abelian() const { return m->symmetry != QCM_SYM_SU2U1; }
    bool allowed(int a, int b, int c) const { return abelian() || triangle(a, b, c); }
    double conj_scale(int lc_s, int rc_s, int spin, int phase) const {
        return abelian() ? 1.0 : conjugate_correction(lc_s, rc_s, spin) * phase;
    }
    void coupling(int j, int jp, int a, int k, int ap, int i, int ip, double scale, double out[4]) const {
        if (abelian()) {
            out[0] = out[1] = out[2] = out[3] = scale;
            return;
        }
        set_coupling(j, std::abs(j - jp), jp, a, k, ap, i, std::abs(i - ip), ip, scale, out);
    }
    bool lskip(int b) const { return m->left_herm[b] < b; }
    bool rskip(int b) const { return m->right_herm[b] < b; }
    int lconj(int b) const { return m->left_herm[b]; }
    int rconj(int b) const { return m->right_herm[b]; }
    int lphase(int b) const { return m->left_phase[b]; }
    int rphase(int b) const { return m->right_phase[b]; }
};

static inline int spin_case(int rs, int cs) {
    if (rs == 2 && cs == 2) return 3;
    if (rs == 2) return 1;
    if (cs == 2) return 2;
    return 0;
}

// ------------------------------------------------------------------ shared building blocks
// Right-paired copy of a left-paired MPS (reshape_left_to_right_new), as gather tiles into `buf`.
static BM plan_reshape_l2r(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& lp, int src_buf,
                           int dst_buf, Stage& st, qcm_plan* P, int64_t& end) {
    PB in_left(phys, left_i, false), out_right(phys, right_i, true);
    BM rp;
    struct Tile { Q ol, orr; int64_t col0, ld, rd; int64_t src; int64_t lds; };
    std::vector<Tile> tiles;
    for (auto& blk : lp.b) {
        size_t r = right_i.position(blk.rc);
        if (r == right_i.size()) continue;
        Q in_r = right_i.d[r].first;
        for (auto& ps : phys.d) {
            size_t l = left_i.position(fuse(blk.lc, neg(ps.first)));
            if (l == left_i.size()) continue;
            Q ol = left_i.d[l].first, orr = fuse(neg(ps.first), in_r);
            if (rp.find(ol, orr) == rp.b.size()) {
                Blk nb;
                nb.lc = ol;
                nb.rc = orr;
                nb.rows = left_i.d[l].second;
                nb.cols = out_right.size(orr);
                rp.insert(nb);
            }
            int64_t ilo = in_left(ps.first, ol), oro = out_right(ps.first, in_r);
            int64_t ld = left_i.d[l].second, rd = right_i.d[r].second;
            for (int64_t ss = 0; ss < ps.second; ++ss)
                tiles.push_back({ol, orr, oro + ss * rd, ld, rd, blk.off + ilo + ss * ld, blk.rows});
        }
    }
    end = rp.assign_offsets(0);
    st.kind = ST_AXPY;
    for (auto& t : tiles) {
        const Blk& d = rp.b[rp.find(t.ol, t.orr)];
        AxpyOut o;
        o.dst_buf = dst_buf;
        o.dst_off = d.off + t.col0 * d.rows;
        o.ldd = d.rows;
        o.rows = t.ld;
        o.cols = t.rd;
        o.t_begin = (int64_t)st.aterm.size();
        st.aterm.push_back({src_buf, t.src, t.lds, 1.0});
        o.t_end = (int64_t)st.aterm.size();
        st.aout.push_back(o);
        P->axpy_bytes += 16.0 * t.ld * t.rd;
    }
    return rp;
}

// K1: T[b1] = A(b1) . rp (BoundaryMPSProduct with gemm_trim_left).
// phases = false: the Hermitian partner L[conj(b1)] is used without the SU(2)
// conjugate correction and bond phase (BoundaryMPSProduct with
// correctConjugate = false, as the zero-site problem builds it).
// align > 1: T's blocks get 16-byte aligned columns (offset and, for blocks of 32
// rows or more, leading dimension rounded up to align elements), so that the
// image epilogue stores T four rows at a time; the padding rows are never read
// into a result (the gather treats a padded source as a pitch x cols run and
// stores only the tile's rows).
static std::vector<BM> plan_k1(const std::vector<BM>& L, const MpoV& W, bool herm, const BM& rp, int rp_buf,
                               const Idx& ref, int t_buf, Stage& st, qcm_plan* P, int64_t& end,
                               bool phases = true, int64_t align = 1) {
    std::vector<BM> T(L.size());
    struct Job { int b1; Q a, l; int64_t a_off, lda; int ta; double scale; int64_t M, K; size_t rpk; };
    std::vector<Job> jobs;
    for (size_t b1 = 0; b1 < L.size(); ++b1) {
        std::vector<Job> Ab;
        bool use_conj = herm && (int)b1 < W.m->row_dim && W.lskip((int)b1);
        if (use_conj) {
            const BM& src = L[W.lconj((int)b1)];
            for (auto& x : src.b) {
                double sc = phases ? W.conj_scale(x.lc.s, x.rc.s, W.lspin((int)b1), W.lphase((int)b1)) : 1.0;
                Ab.push_back({(int)b1, x.lc, x.rc, x.off, x.rows, 0, sc, x.rows, x.cols, 0});
            }
        } else {
            for (auto& x : L[b1].b) Ab.push_back({(int)b1, x.rc, x.lc, x.off, x.rows, 1, 1.0, x.cols, x.rows, 0});
        }
        std::stable_sort(Ab.begin(), Ab.end(), [](const Job& p, const Job& q) {
            return p.a > q.a || (p.a == q.a && p.l > q.l);
        });
        for (auto& j : Ab) {
            if (!ref.has(j.a)) continue;
            size_t it = rp.left_lower_bound(j.l);
            for (; it < rp.b.size() && rp.b[it].lc == j.l; ++it) {
                Blk nb;
                nb.lc = j.a;
                nb.rc = rp.b[it].rc;
                nb.rows = j.M;
                nb.cols = rp.b[it].cols;
                if (T[b1].find(nb.lc, nb.rc) != T[b1].b.size()) throw std::runtime_error("duplicate T block");
                T[b1].insert(nb);
                Job jj = j;
                jj.rpk = it;
                jobs.push_back(jj);
            }
        }
    }
    int64_t base = 0;
    for (auto& t : T) base = t.assign_offsets_aligned(base, align);
    end = base;
    st.kind = ST_GEMM;
    for (auto& j : jobs) {
        const Blk& rb = rp.b[j.rpk];
        const Blk& c = T[j.b1].b[T[j.b1].find(j.a, rb.rc)];
        GemmOut o;
        o.c_buf = t_buf;
        o.c_off = c.off;
        o.ldc = c.pitch();
        o.vec_store = align >= 4 && c.off % 4 == 0 && c.pitch() % 4 == 0 ? 1 : 0;
        o.M = c.rows;
        o.N = c.cols;
        o.s_begin = (int64_t)st.gseg.size();
        GemmSeg s;
        s.a_buf = QCM_BUF_LEFT;
        s.ta = j.ta;
        s.a_off = j.a_off;
        s.lda = j.lda;
        s.b_buf = rp_buf;
        s.tb = 0;
        s.b_off = rb.off;
        s.ldb = rb.rows;
        s.K = j.K;
        s.alpha = j.scale;
        if (rb.rows != j.K) throw std::runtime_error("K1 inner dimension mismatch");
        st.gseg.push_back(s);
        o.s_end = (int64_t)st.gseg.size();
        st.gout.push_back(o);
        P->gemm_flops += 2.0 * c.rows * c.cols * j.K;
    }
    return T;
}

// K2: contr[b2] = sum_{b1,op} couplings x stripes of T[b1]  (lbtm_kernel).
// prov (optional): per emitted term, in aterm order, the MPO term it comes from
// (index into term_op/term_scale) and its coefficient per unit of that term's scale.
// alloc_all: also the blocks the abelian kernel allocates whether or not a term
// writes them (lbtm_kernel_allocate, ct/abelian/apply_op.hpp:23-66: for every
// (b1, operator) of the column with a non-empty T[b1], one block per right
// sector, at the operator's and T's constant charge shifts); they stay zero but
// are part of a boundary's layout.
static std::vector<BM> plan_k2(const std::vector<BM>& T, const MpoV& W, const std::vector<int>& b2list,
                               const Idx& right_i, const Idx& out_left_i, const PB& in_right_pb,
                               const PB& out_left_pb, int t_buf, int c_buf, Stage& st, qcm_plan* P, int64_t& end,
                               std::vector<std::pair<int32_t, double>>* prov = nullptr, bool alloc_all = false) {
    const qcm_mpo_t* m = W.m;
    std::vector<BM> C(m->col_dim);
    // the terms of one b2 column with their tile keys, sorted (stably) by key
    // afterwards.  key = position of out_l in out_left_i (16 bits), of out_r in
    // right_i (16 bits), row offset (32 bits): ascending keys are the reference's
    // block order (both indices descend) with row offsets ascending.
    struct KeyedTerm { uint64_t key; int64_t src_off; double alpha; int32_t rows, cols, tt, lds; };
    if (out_left_i.size() >= (1u << 16) || right_i.size() >= (1u << 16))
        throw std::runtime_error("too many sectors for the K2 planner");
    for (int b2 : b2list)
        if (b2 < 0 || b2 >= m->col_dim) throw std::runtime_error("b2 out of range");
    for (int e = 0; e < m->col_ptr[m->col_dim]; ++e)
        if (m->row_of[e] >= (int)T.size()) throw std::runtime_error("mpo row beyond boundary aux dimension");
    // The MPO elements of one b2 column, [e0, e1): the contr blocks they need and
    // their keyed terms (independent of every other task).
    struct BlkNeed { Q lc, rc; int64_t rows, cols; };
    struct TaskOut { std::vector<KeyedTerm> terms; std::vector<BlkNeed> blocks; double flops = 0.0; };
    auto column = [&](int b2, int e0, int e1, TaskOut& out) {
        int ap = W.rspin(b2);
        for (int e = e0; e < e1; ++e) {
            int b1 = m->row_of[e];
            int a = W.lspin(b1);
            for (int tt = m->term_ptr[e]; tt < m->term_ptr[e + 1]; ++tt) {
                int op = m->term_op[tt];
                double scale = m->term_scale[tt];
                int k = m->op_spin[op];
                if (alloc_all && !T[b1].b.empty() && m->op_blk_ptr[op] < m->op_blk_ptr[op + 1]) {
                    const int w0 = m->op_blk_ptr[op];
                    const Q op_delta = fuse(Q(m->blk_q[4 * w0 + 2], m->blk_q[4 * w0 + 3]),
                                            neg(Q(m->blk_q[4 * w0], m->blk_q[4 * w0 + 1])));
                    const Q t_delta = fuse(T[b1].b[0].rc, neg(T[b1].b[0].lc));
                    const Q total = fuse(op_delta, neg(t_delta));
                    for (auto& rs : right_i.d) {
                        const Q out_l = fuse(rs.first, total);
                        const size_t pl = out_left_i.position(out_l);
                        if (pl != out_left_i.size()) out.blocks.push_back({out_l, rs.first, out_left_i.d[pl].second, rs.second});
                    }
                }
                for (auto& tb : T[b1].b) {
                    Q lc = tb.lc, rc = tb.rc, mc = tb.rc;
                    int64_t l_size = tb.rows;
                    const int64_t ldt = tb.pitch();
                    for (int wb = m->op_blk_ptr[op]; wb < m->op_blk_ptr[op + 1]; ++wb) {
                        Q pin(m->blk_q[4 * wb], m->blk_q[4 * wb + 1]), pout(m->blk_q[4 * wb + 2], m->blk_q[4 * wb + 3]);
                        Q out_r = fuse(rc, pin);
                        size_t rb = right_i.position(out_r);
                        if (rb == right_i.size()) continue;
                        Q out_l = fuse(lc, pout);
                        if (!W.allowed(out_r.s, ap, out_l.s)) continue;
                        const size_t pl = out_left_i.position(out_l);
                        if (pl == out_left_i.size()) continue;
                        int64_t r_size = right_i.d[rb].second;
                        if (l_size >= (int64_t(1) << 31) || r_size >= (int64_t(1) << 31))
                            throw std::runtime_error("block larger than 2^31 elements");
                        out.blocks.push_back({out_l, out_r, out_left_i.d[pl].second, r_size});
                        int i = lc.s, ip = out_l.s, j = mc.s, jp = out_r.s;
                        double cpl[4];
                        W.coupling(j, jp, a, k, ap, i, ip, scale, cpl);
                        int64_t iro = in_right_pb(pin, out_r), olo = out_left_pb(pout, lc);
                        for (int en = m->blk_ent_ptr[wb]; en < m->blk_ent_ptr[wb + 1]; ++en) {
                            int ss1 = m->ent[4 * en], ss2 = m->ent[4 * en + 1];
                            double alfa = m->ent_coeff[en] * cpl[spin_case(m->ent[4 * en + 2], m->ent[4 * en + 3])];
                            if (alfa == 0.0) continue;
                            const uint64_t key = ((uint64_t)pl << 48) | ((uint64_t)rb << 32) |
                                                 (uint64_t)(uint32_t)(olo + ss2 * l_size);
                            out.terms.push_back({key, tb.off + (iro + (int64_t)ss1 * r_size) * ldt, alfa,
                                                 (int32_t)l_size, (int32_t)r_size, tt, (int32_t)ldt});
                            out.flops += 2.0 * l_size * r_size;
                        }
                    }
                }
            }
        }
    };
    // tasks: each b2 column cut into runs of at most 8 MPO elements (the Hamiltonian's
    // complementary-operator columns hold hundreds), planned by all host threads
    struct Task { size_t col; int e0, e1; };
    std::vector<Task> tasks;
    std::vector<size_t> task_begin(b2list.size() + 1, 0);
    for (size_t i = 0; i < b2list.size(); ++i) {
        task_begin[i] = tasks.size();
        const int b2 = b2list[i];
        for (int e = m->col_ptr[b2]; e < m->col_ptr[b2 + 1]; e += 8)
            tasks.push_back({i, e, std::min(e + 8, m->col_ptr[b2 + 1])});
    }
    task_begin[b2list.size()] = tasks.size();
    std::vector<TaskOut> tout(tasks.size());
    // per column: pointers to its terms (in the tasks' own lists, task order),
    // stably ordered by tile key
    std::vector<std::vector<const KeyedTerm*>> ord(b2list.size());
    std::vector<double> fl(b2list.size(), 0.0);
    auto parallel = [&](size_t n, const std::function<void(size_t)>& f) {
        std::atomic<size_t> next{0};
        std::mutex err_mu;
        std::string err;
        auto worker = [&]() {
            for (;;) {
                const size_t i = next.fetch_add(1);
                if (i >= n) return;
                try {
                    f(i);
                } catch (const std::exception& ex) {
                    std::lock_guard<std::mutex> g(err_mu);
                    if (err.empty()) err = ex.what();
                }
            }
        };
        const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; ++t) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
        if (!err.empty()) throw std::runtime_error(err);
    };
    parallel(tasks.size(), [&](size_t ti) { column(b2list[tasks[ti].col], tasks[ti].e0, tasks[ti].e1, tout[ti]); });
    // per column: its blocks, and its terms stably ordered by key.  A column has few
    // distinct keys (its output tiles) and many terms per key, so the terms are
    // grouped by key through a hash table, the distinct keys sorted, and every group
    // laid out in task and position order -- the order a stable sort of the
    // concatenated task lists by key gives
    parallel(b2list.size(), [&](size_t i) {
        const int b2 = b2list[i];
        size_t nt = 0;
        for (size_t ti = task_begin[i]; ti < task_begin[i + 1]; ++ti) {
            nt += tout[ti].terms.size();
            fl[i] += tout[ti].flops;
            for (const BlkNeed& bn : tout[ti].blocks)
                if (C[b2].find(bn.lc, bn.rc) == C[b2].b.size()) {
                    Blk nb;
                    nb.lc = bn.lc;
                    nb.rc = bn.rc;
                    nb.rows = bn.rows;
                    nb.cols = bn.cols;
                    C[b2].insert(nb);
                }
            std::vector<BlkNeed>().swap(tout[ti].blocks);
        }
        std::unordered_map<uint64_t, uint32_t> gid;
        gid.reserve(1024);
        std::vector<uint32_t> g(nt), cnt;
        std::vector<uint64_t> gkey;
        size_t k = 0;
        for (size_t ti = task_begin[i]; ti < task_begin[i + 1]; ++ti)
            for (const KeyedTerm& x : tout[ti].terms) {
                auto it = gid.find(x.key);
                if (it == gid.end()) {
                    it = gid.emplace(x.key, (uint32_t)gkey.size()).first;
                    gkey.push_back(x.key);
                    cnt.push_back(0);
                }
                g[k++] = it->second;
                ++cnt[it->second];
            }
        std::vector<uint32_t> rank(gkey.size());
        for (size_t q = 0; q < rank.size(); ++q) rank[q] = (uint32_t)q;
        std::sort(rank.begin(), rank.end(), [&](uint32_t a, uint32_t b) { return gkey[a] < gkey[b]; });
        std::vector<size_t> pos(gkey.size());
        size_t acc = 0;
        for (uint32_t r : rank) { pos[r] = acc; acc += cnt[r]; }
        std::vector<const KeyedTerm*>& o = ord[i];
        o.resize(nt);
        k = 0;
        for (size_t ti = task_begin[i]; ti < task_begin[i + 1]; ++ti)
            for (const KeyedTerm& x : tout[ti].terms) o[pos[g[k++]]++] = &x;
    });
    int64_t base = 0;
    for (auto& c : C) base = c.assign_offsets(base);
    end = base;
    st.kind = ST_AXPY;
    // emit in b2 order: count each column's tiles, then every column fills its own
    // precomputed range of the output and term tables (in parallel)
    std::vector<size_t> ntile(b2list.size(), 0);
    parallel(b2list.size(), [&](size_t i) {
        const std::vector<const KeyedTerm*>& o = ord[i];
        size_t n = 0;
        for (size_t a = 0; a < o.size(); ++a)
            if (a == 0 || o[a]->key != o[a - 1]->key) ++n;
        ntile[i] = n;
    });
    std::vector<size_t> obase(b2list.size() + 1, st.aout.size()), tbase(b2list.size() + 1, st.aterm.size());
    for (size_t i = 0; i < b2list.size(); ++i) {
        obase[i + 1] = obase[i] + ntile[i];
        tbase[i + 1] = tbase[i] + ord[i].size();
    }
    st.aout.resize(obase[b2list.size()]);
    st.aterm.resize(tbase[b2list.size()]);
    if (prov) prov->assign(st.aterm.size(), {0, 0.0});
    std::vector<double> bytes(b2list.size(), 0.0);
    parallel(b2list.size(), [&](size_t i) {
        const int b2 = b2list[i];
        const BM& cb = C[b2];
        std::vector<const KeyedTerm*>& ov = ord[i];
        size_t oi = obase[i], ti = tbase[i];
        for (size_t a = 0; a < ov.size();) {
            size_t b = a + 1;
            while (b < ov.size() && ov[b]->key == ov[a]->key) ++b;   // equal keys: one tile
            const uint64_t key = ov[a]->key;
            const Q out_l = out_left_i.d[key >> 48].first, out_r = right_i.d[(key >> 32) & 0xFFFFu].first;
            const Blk& d = cb.b[cb.find(out_l, out_r)];
            const KeyedTerm& last = *ov[b - 1];
            AxpyOut& o = st.aout[oi++];
            o.dst_buf = c_buf;
            o.dst_off = d.off + (int64_t)(uint32_t)(key & 0xFFFFFFFFu);
            o.ldd = d.rows;
            o.rows = last.rows;
            o.cols = last.cols;
            o.t_begin = (int64_t)ti;
            for (size_t k = a; k < b; ++k) {
                const KeyedTerm& x = *ov[k];
                if (prov) (*prov)[ti] = {x.tt, x.alpha / m->term_scale[x.tt]};
                st.aterm[ti++] = {t_buf, x.src_off, x.lds, x.alpha};
            }
            o.t_end = (int64_t)ti;
            bytes[i] += 8.0 * o.rows * o.cols * (double)(b - a + 1);
            a = b;
        }
        std::vector<const KeyedTerm*>().swap(ov);
    });
    for (size_t i = 0; i < b2list.size(); ++i) {
        P->axpy_flops += fl[i];
        P->axpy_bytes += bytes[i];
    }
    return C;
}

// Split-K for grouped GEMM outputs with long segment lists: every output with
// more than `max_segs` segments is cut into parts of at most `max_segs`
// segments; each part writes its partial tile to `buf` (dense, ld = M) and a
// gather stage sums the parts into the output in part order.  Outputs that are
// short enough keep writing the output directly.  Results stay independent of
// scheduling; the FP64 sums differ from the unsplit order only by rounding.
static void split_k(Stage& g, int buf, int64_t base, int64_t max_segs, Stage& red, int64_t& end) {
    std::vector<GemmOut> outs;
    red.kind = ST_AXPY;
    int64_t off = base;
    for (const GemmOut& o : g.gout) {
        int64_t nseg = o.s_end - o.s_begin;
        if (nseg <= max_segs) {
            outs.push_back(o);
            continue;
        }
        AxpyOut r;
        r.dst_buf = o.c_buf;
        r.dst_off = o.c_off;
        r.ldd = o.ldc;
        r.rows = o.M;
        r.cols = o.N;
        r.t_begin = (int64_t)red.aterm.size();
        for (int64_t s0 = o.s_begin; s0 < o.s_end; s0 += max_segs) {
            GemmOut p = o;
            p.c_buf = buf;
            p.c_off = off;
            p.ldc = o.M;
            p.s_begin = s0;
            p.s_end = std::min(o.s_end, s0 + max_segs);
            outs.push_back(p);
            red.aterm.push_back({buf, off, o.M, 1.0});
            off += o.M * o.N;
        }
        r.t_end = (int64_t)red.aterm.size();
        red.aout.push_back(r);
    }
    g.gout.swap(outs);
    end = off;
}

static void finalize_boundary_layout(qcm_plan* P, std::vector<BM>& out) {
    int64_t base = 0;
    P->out_blk_ptr.assign(1, 0);
    for (auto& bm : out) {
        base = bm.assign_offsets(base);
        for (auto& b : bm.b) P->out_blocks.push_back(b);
        P->out_blk_ptr.push_back((int32_t)P->out_blocks.size());
    }
    P->out_elems = base;
}

// ------------------------------------------------------------------ plan kinds
// The parts of the contr blocks that K3 reads but no K2 tile writes must be
// zero.  Instead of clearing the whole contr arena, append zero-term output
// tiles (written as zeros by the gather executors) covering exactly those
// parts: per block, between consecutive column breakpoints of its tiles, the
// row ranges no tile covers.  Blocks K3 never reads are left unwritten.
static void add_zero_tiles(Stage& k2, const Stage& k3, int32_t buf) {
    struct B { int64_t off, ld, cols; };
    std::vector<B> blocks;
    for (const GemmSeg& g : k3.gseg)
        if (g.a_buf == buf && g.ta == 0) blocks.push_back({g.a_off, g.lda, g.K});
    std::sort(blocks.begin(), blocks.end(), [](const B& x, const B& y) { return x.off < y.off; });
    blocks.erase(std::unique(blocks.begin(), blocks.end(), [](const B& x, const B& y) { return x.off == y.off; }),
                 blocks.end());
    struct T { int64_t r0, c0, rows, cols; };
    std::vector<std::vector<T>> in(blocks.size());
    for (const AxpyOut& a : k2.aout) {
        if (a.dst_buf != buf) continue;
        auto it = std::upper_bound(blocks.begin(), blocks.end(), a.dst_off,
                                   [](int64_t o, const B& b) { return o < b.off; });
        if (it == blocks.begin()) continue;
        --it;
        const int64_t rel = a.dst_off - it->off;
        if (rel >= it->ld * it->cols) continue;  // a block K3 does not read
        if (a.ldd != it->ld) throw std::runtime_error("contr tile does not match its block");
        in[it - blocks.begin()].push_back({rel % it->ld, rel / it->ld, a.rows, a.cols});
    }
    const int64_t t_at = (int64_t)k2.aterm.size();
    for (size_t bi = 0; bi < blocks.size(); ++bi) {
        const B& b = blocks[bi];
        std::vector<int64_t> cut{0, b.cols};
        for (const T& t : in[bi]) { cut.push_back(t.c0); cut.push_back(t.c0 + t.cols); }
        std::sort(cut.begin(), cut.end());
        cut.erase(std::unique(cut.begin(), cut.end()), cut.end());
        for (size_t k = 0; k + 1 < cut.size(); ++k) {
            const int64_t ca = cut[k], cb = cut[k + 1];
            if (ca >= b.cols) break;
            std::vector<std::pair<int64_t, int64_t>> rr;
            for (const T& t : in[bi])
                if (t.c0 <= ca && cb <= t.c0 + t.cols) rr.push_back({t.r0, t.r0 + t.rows});
            std::sort(rr.begin(), rr.end());
            int64_t r = 0;
            auto emit = [&](int64_t r_lo, int64_t r_hi) {
                if (r_hi <= r_lo) return;
                AxpyOut z;
                z.dst_buf = buf;
                z.dst_off = b.off + r_lo + ca * b.ld;
                z.ldd = b.ld;
                z.rows = r_hi - r_lo;
                z.cols = cb - ca;
                z.t_begin = z.t_end = t_at;
                k2.aout.push_back(z);
            };
            for (const auto& iv : rr) {
                emit(r, iv.first);
                r = std::max(r, iv.second);
            }
            emit(r, b.ld);
        }
    }
}

static qcm_plan* build_sigma(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& psi,
                             const std::vector<BM>& L, const std::vector<BM>& R, const MpoV& W, bool herm,
                             int64_t split_k_segs = 32, int64_t dense_min_terms = 64, int n_tile_max = 128,
                             bool k1_resident = kAResident) {
    auto* P = new qcm_plan();
    P->kind = PK_SIGMA;
    const qcm_mpo_t* m = W.m;
    if ((int)L.size() != m->row_dim || (int)R.size() != m->col_dim)
        throw std::runtime_error("boundary aux dimensions do not match the MPO");
    // output sigma: same layout as psi
    int64_t psi_end = 0;
    for (auto& b : psi.b) psi_end = std::max(psi_end, b.off + b.rows * b.cols);
    P->out_elems = psi_end;

    Idx out_left_i = index_product(phys, left_i);
    Idx rib = right_i;
    common_subset(out_left_i, rib);
    PB out_left_pb(phys, left_i, false), in_right_pb(phys, right_i, true);

    Stage z0; z0.kind = ST_ZERO; z0.zbuf = QCM_BUF_S0;
    Stage s0; int64_t rp_end = 0;
    BM rp = plan_reshape_l2r(phys, left_i, right_i, psi, QCM_BUF_KET, QCM_BUF_S0, s0, P, rp_end);
    z0.zlen = rp_end;
    Idx ref;
    for (auto& b : rp.b) ref.d.push_back({b.lc, b.rows});
    Stage s1; int64_t t_end = 0;
    std::vector<BM> T = plan_k1(L, W, herm, rp, QCM_BUF_S0, ref, QCM_BUF_S1, s1, P, t_end, true, kTAlign);
    std::vector<int> b2list;
    for (int b2 = 0; b2 < m->col_dim; ++b2) b2list.push_back(b2);
    Stage s2; int64_t c_end = 0;
    std::vector<BM> C = plan_k2(T, W, b2list, right_i, out_left_i, in_right_pb, out_left_pb, QCM_BUF_S1,
                                QCM_BUF_S2, s2, P, c_end);
    Stage z2; z2.kind = ST_ZERO; z2.zbuf = QCM_BUF_S2; z2.zlen = c_end;
    // K3: sigma(al,al) = sum_b2 contr[b2](al,ar) . R'[b2](ar,al)  (gemm_trim)
    Stage s3; s3.kind = ST_GEMM;
    for (auto& ob : psi.b) {
        if (!(ob.lc == ob.rc)) throw std::runtime_error("psi layout is not block diagonal (left-paired)");
        Q al = ob.lc;
        GemmOut o;
        o.c_buf = QCM_BUF_OUT;
        o.c_off = ob.off;
        o.ldc = ob.rows;
        o.M = ob.rows;
        o.N = ob.cols;
        o.s_begin = (int64_t)s3.gseg.size();
        for (int b2 = 0; b2 < m->col_dim; ++b2) {
            const BM& cb = C[b2];
            size_t it = cb.left_lower_bound(al);
            for (; it < cb.b.size() && cb.b[it].lc == al; ++it) {
                const Blk& a = cb.b[it];
                Q ar = a.rc;
                GemmSeg s;
                s.a_buf = QCM_BUF_S2; s.ta = 0; s.a_off = a.off; s.lda = a.rows; s.K = a.cols;
                if (herm && W.rskip(b2)) {
                    const BM& rs = R[W.rconj(b2)];
                    size_t k = rs.find(al, ar);
                    if (k == rs.b.size()) continue;
                    s.b_buf = QCM_BUF_RIGHT; s.tb = 1; s.b_off = rs.b[k].off; s.ldb = rs.b[k].rows;
                    s.alpha = W.conj_scale(ar.s, al.s, W.rspin(b2), W.rphase(W.rconj(b2)));
                    if (rs.b[k].cols != a.cols || rs.b[k].rows != ob.cols)
                        throw std::runtime_error("K3 dimension mismatch (adjoint)");
                } else {
                    const BM& rs = R[b2];
                    size_t k = rs.find(ar, al);
                    if (k == rs.b.size()) continue;
                    s.b_buf = QCM_BUF_RIGHT; s.tb = 0; s.b_off = rs.b[k].off; s.ldb = rs.b[k].rows;
                    s.alpha = 1.0;
                    if (rs.b[k].rows != a.cols || rs.b[k].cols != ob.cols)
                        throw std::runtime_error("K3 dimension mismatch");
                }
                if (a.rows != ob.rows) throw std::runtime_error("K3 row mismatch");
                s3.gseg.push_back(s);
                P->gemm_flops += 2.0 * ob.rows * ob.cols * a.cols;
            }
        }
        o.s_end = (int64_t)s3.gseg.size();
        s3.gout.push_back(o);
    }
    // split-K over the MPO bond sum: partial tiles in scratch 1 (T is dead after K2)
    Stage s4;
    int64_t part_end = 0;
    split_k(s3, QCM_BUF_S1, 0, split_k_segs, s4, part_end);
    for (auto& a : s4.aout) P->axpy_bytes += 8.0 * a.rows * a.cols * (double)(a.t_end - a.t_begin + 1);
    P->scratch[0] = rp_end;
    P->scratch[1] = std::max(t_end, part_end);
    P->scratch[2] = c_end;
    add_zero_tiles(s2, s3, QCM_BUF_S2);
    z2.zlen = 0;  // the zero tiles of K2 clear what K3 reads; the rest of contr is never read
    build_image_tables(s1, s1.img, n_tile_max, k1_resident);
    build_image_tables(s3, s3.img, n_tile_max, false);
    axpy_components(s2, s2.comp_root);
    build_dense_groups(s2, dense_min_terms, s2.img, s2.heavy);
    P->image_bytes = std::max(std::max(s1.img.bytes, s3.img.bytes), s2.img.bytes);
    P->stages.push_back(std::move(z0));
    P->stages.push_back(std::move(s0));
    P->stages.push_back(std::move(s1));
    P->stages.push_back(std::move(z2));
    P->stages.push_back(std::move(s2));
    P->stages.push_back(std::move(s3));
    if (!s4.aout.empty()) P->stages.push_back(std::move(s4));
    return P;
}

// Zero-site problem (zerosite_hamil_lbtm_kernel, ct/non-abelian/zero_site_hamil.hpp:44-79):
// the bond matrix C between two sites, the left boundary L and the right boundary R
// of that bond, the MPO tensors either side of it (Wl: its columns are the bond,
// Wr: its rows are the bond).  sigma(al,al) = sum_b op(L[b])^T C (al,ar) . R'[b](ar,al)
// with, for the bonds Wr marks as Hermitian partners, L[conj b] and R[conj b]^T in
// place of L[b]^T and R[b], both without phases (the reference passes
// correctConjugate = false and unit scales).  Stages: K1 (T[b] = op(L[b]) C into
// S1), K3 (sigma into OUT, split-K partials in S0), the split-K sum.
static qcm_plan* build_zerosite(const BM& bond, const std::vector<BM>& L, const std::vector<BM>& R,
                                const MpoV& Wl, const MpoV& Wr, bool herm, int64_t split_k_segs = 32) {
    auto* P = new qcm_plan();
    P->kind = PK_SIGMA;
    const int nb = Wr.m->row_dim;
    if (Wl.m->col_dim != nb) throw std::runtime_error("MPO tensors do not share the bond");
    if ((int)L.size() != nb || (int)R.size() != nb)
        throw std::runtime_error("boundary aux dimensions do not match the bond");
    int64_t c_end = 0;
    for (auto& b : bond.b) {
        if (!(b.lc == b.rc)) throw std::runtime_error("bond matrix is not block diagonal");
        c_end = std::max(c_end, b.off + b.rows * b.cols);
    }
    P->out_elems = c_end;
    Idx ref;
    for (auto& b : bond.b) ref.d.push_back({b.lc, b.rows});
    Stage s1; int64_t t_end = 0;
    std::vector<BM> T = plan_k1(L, Wr, herm, bond, QCM_BUF_KET, ref, QCM_BUF_S1, s1, P, t_end, false);
    Stage s3; s3.kind = ST_GEMM;
    for (auto& ob : bond.b) {
        Q al = ob.lc;
        GemmOut o;
        o.c_buf = QCM_BUF_OUT;
        o.c_off = ob.off;
        o.ldc = ob.rows;
        o.M = ob.rows;
        o.N = ob.cols;
        o.s_begin = (int64_t)s3.gseg.size();
        for (int b = 0; b < nb; ++b) {
            const BM& tb = T[b];
            size_t it = tb.left_lower_bound(al);
            for (; it < tb.b.size() && tb.b[it].lc == al; ++it) {
                const Blk& a = tb.b[it];
                Q ar = a.rc;
                GemmSeg g;
                g.a_buf = QCM_BUF_S1; g.ta = 0; g.a_off = a.off; g.lda = a.rows; g.K = a.cols;
                g.alpha = 1.0;
                if (herm && Wr.lskip(b)) {
                    const BM& rs = R[Wl.rconj(b)];
                    size_t k = rs.find(al, ar);
                    if (k == rs.b.size()) continue;
                    g.b_buf = QCM_BUF_RIGHT; g.tb = 1; g.b_off = rs.b[k].off; g.ldb = rs.b[k].rows;
                    if (rs.b[k].cols != a.cols || rs.b[k].rows != ob.cols)
                        throw std::runtime_error("zero-site dimension mismatch (adjoint)");
                } else {
                    const BM& rs = R[b];
                    size_t k = rs.find(ar, al);
                    if (k == rs.b.size()) continue;
                    g.b_buf = QCM_BUF_RIGHT; g.tb = 0; g.b_off = rs.b[k].off; g.ldb = rs.b[k].rows;
                    if (rs.b[k].rows != a.cols || rs.b[k].cols != ob.cols)
                        throw std::runtime_error("zero-site dimension mismatch");
                }
                if (a.rows != ob.rows) throw std::runtime_error("zero-site row mismatch");
                s3.gseg.push_back(g);
                P->gemm_flops += 2.0 * ob.rows * ob.cols * a.cols;
            }
        }
        o.s_end = (int64_t)s3.gseg.size();
        s3.gout.push_back(o);
    }
    Stage s4;
    int64_t part_end = 0;
    split_k(s3, QCM_BUF_S0, 0, split_k_segs, s4, part_end);
    for (auto& a : s4.aout) P->axpy_bytes += 8.0 * a.rows * a.cols * (double)(a.t_end - a.t_begin + 1);
    P->scratch[0] = part_end;
    P->scratch[1] = t_end;
    P->scratch[2] = 0;
    build_image_tables(s1, s1.img);
    build_image_tables(s3, s3.img);
    P->image_bytes = std::max(s1.img.bytes, s3.img.bytes);
    P->stages.push_back(std::move(s1));
    P->stages.push_back(std::move(s3));
    if (!s4.aout.empty()) P->stages.push_back(std::move(s4));
    return P;
}

// Diagonal of H_eff (SU2::diagonal_hamiltonian + lbtm_diag_kernel,
// ct/non-abelian/h_diag.hpp:13-158) in the ket's left-paired layout.  Every L[b1]
// and R[b2] is read as given (the reference uses no Hermitian partners here).  A
// contribution -- b2, b1 of its column, a term, a phys charge p with lc = c - p,
// a diagonal operator entry (ss, ss) -- adds alfa * diag(L[b1](lc,lc)) (x)
// diag(R[b2](c,c)) to the ld rows of (p, ss, lc) in every column of block (c, c),
// when R[b2] holds (c, c).  Stages: the diagonals of the boundary blocks as dense
// vectors (one strided 1 x n tile per block: L into S0, R into S1), a clear of
// OUT, then one K = 1 product per contribution, summed per (block, row stripe),
// split-K partials in S2 and their sum.
static qcm_plan* build_diag(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& psi,
                            const std::vector<BM>& L, const std::vector<BM>& R, const MpoV& W,
                            int64_t split_k_segs = 32) {
    auto* P = new qcm_plan();
    P->kind = PK_DIAG;
    const qcm_mpo_t* m = W.m;
    if ((int)L.size() != m->row_dim || (int)R.size() != m->col_dim)
        throw std::runtime_error("boundary aux dimensions do not match the MPO");
    int64_t psi_end = 0;
    for (auto& b : psi.b) psi_end = std::max(psi_end, b.off + b.rows * b.cols);
    P->out_elems = psi_end;
    Idx out_left_i = index_product(phys, left_i);
    Idx rib = right_i;
    common_subset(out_left_i, rib);
    PB left_pb(phys, left_i, false);
    // diagonals of the square charge-diagonal boundary blocks
    Stage sx; sx.kind = ST_AXPY;
    // (bond index, charge) -> (offset, length) of the diagonal vector
    std::vector<std::map<std::pair<int, int>, std::pair<int64_t, int64_t>>> dl(L.size()), dr(R.size());
    int64_t l_end = 0, r_end = 0;
    auto diag_tiles = [&](const std::vector<BM>& B, int src, int dst, int64_t& end,
                          std::vector<std::map<std::pair<int, int>, std::pair<int64_t, int64_t>>>& where) {
        for (size_t b = 0; b < B.size(); ++b)
            for (const Blk& x : B[b].b) {
                if (!(x.lc == x.rc) || x.rows != x.cols || x.rows == 0) continue;
                AxpyOut o;
                o.dst_buf = dst;
                o.dst_off = end;
                o.ldd = 1;
                o.rows = 1;
                o.cols = x.rows;
                o.t_begin = (int64_t)sx.aterm.size();
                sx.aterm.push_back({src, x.off, x.rows + 1, 1.0});
                o.t_end = (int64_t)sx.aterm.size();
                sx.aout.push_back(o);
                where[b][{x.lc.n, x.lc.s}] = {end, x.rows};
                end += x.rows;
            }
    };
    diag_tiles(L, QCM_BUF_LEFT, QCM_BUF_S0, l_end, dl);
    diag_tiles(R, QCM_BUF_RIGHT, QCM_BUF_S1, r_end, dr);
    Stage z; z.kind = ST_ZERO; z.zbuf = QCM_BUF_OUT; z.zlen = psi_end;
    // one output per (psi block, phys charge, diagonal entry row, lc) stripe
    Stage sg; sg.kind = ST_GEMM;
    struct Contrib { int b1, b2, tt, ss; double alfa; };
    for (const Blk& ob : psi.b) {
        if (!(ob.lc == ob.rc)) throw std::runtime_error("psi layout is not block diagonal (left-paired)");
        const Q c = ob.lc;
        if (!rib.has(c) || !out_left_i.has(c)) continue;
        if (out_left_i.size_of(c) != ob.rows || rib.size_of(c) != ob.cols)
            throw std::runtime_error("psi block does not match the product index");
        const int jp = c.s, ip = c.s;
        for (auto& pp : phys.d) {
            const Q pc = pp.first;
            const Q lin = fuse(c, neg(pc));
            const size_t l = left_i.position(lin);
            if (l == left_i.size()) continue;
            const int64_t ld = left_i.d[l].second;
            const int64_t loff = left_pb(pc, lin);
            // contributions grouped by the operator entry's row ss
            std::map<int, std::vector<Contrib>> per_ss;
            for (int b2 = 0; b2 < m->col_dim; ++b2) {
                auto rit = dr[b2].find({c.n, c.s});
                if (rit == dr[b2].end()) continue;
                if (rit->second.second < ob.cols) throw std::runtime_error("right boundary block smaller than psi's");
                const int ap = W.rspin(b2);
                for (int e = m->col_ptr[b2]; e < m->col_ptr[b2 + 1]; ++e) {
                    const int b1 = m->row_of[e];
                    auto lit = dl[b1].find({lin.n, lin.s});
                    if (lit == dl[b1].end()) continue;
                    if (lit->second.second < ld) throw std::runtime_error("left boundary block smaller than psi's");
                    const int a = W.lspin(b1);
                    const int i = lin.s, j = lin.s;
                    for (int tt = m->term_ptr[e]; tt < m->term_ptr[e + 1]; ++tt) {
                        const int op = m->term_op[tt];
                        const int k = m->op_spin[op];
                        const double pref = std::sqrt((ip + 1.0) * (j + 1.0) / ((i + 1.0) * (jp + 1.0))) *
                                            m->term_scale[tt];
                        const double c0 = W.abelian() ? m->term_scale[tt]
                                                      : pref * mod_coupling(j, std::abs(j - jp), jp, a, k, ap, i,
                                                                            std::abs(i - ip), ip);
                        const double c1 = W.abelian() ? m->term_scale[tt]
                                                      : pref * mod_coupling(j, 2, jp, a, k, ap, i, 2, ip);
                        for (int wb = m->op_blk_ptr[op]; wb < m->op_blk_ptr[op + 1]; ++wb) {
                            Q pin(m->blk_q[4 * wb], m->blk_q[4 * wb + 1]), pout(m->blk_q[4 * wb + 2], m->blk_q[4 * wb + 3]);
                            if (!(pin == pc) || !(pin == pout)) continue;
                            for (int en = m->blk_ent_ptr[wb]; en < m->blk_ent_ptr[wb + 1]; ++en) {
                                const int ss1 = m->ent[4 * en], ss2 = m->ent[4 * en + 1];
                                if (ss1 != ss2) continue;
                                const double alfa = m->ent_coeff[en] * (m->ent[4 * en + 2] == 2 ? c1 : c0);
                                if ((int64_t)(ss1 + 1) * ld > pp.second * ld) throw std::runtime_error("operator entry beyond phys sector");
                                per_ss[ss1].push_back({b1, b2, tt, ss1, alfa});
                            }
                        }
                    }
                }
            }
            for (auto& [ss, list] : per_ss) {
                GemmOut o;
                o.c_buf = QCM_BUF_OUT;
                o.c_off = ob.off + loff + (int64_t)ss * ld;
                o.ldc = ob.rows;
                o.M = ld;
                o.N = ob.cols;
                if (loff + (int64_t)(ss + 1) * ld > ob.rows) throw std::runtime_error("diagonal stripe beyond psi block");
                o.s_begin = (int64_t)sg.gseg.size();
                for (const Contrib& q : list) {
                    GemmSeg g;
                    g.a_buf = QCM_BUF_S0; g.ta = 0; g.a_off = dl[q.b1][{lin.n, lin.s}].first; g.lda = ld;
                    g.b_buf = QCM_BUF_S1; g.tb = 0; g.b_off = dr[q.b2][{c.n, c.s}].first; g.ldb = 1;
                    g.K = 1;
                    g.alpha = q.alfa;
                    sg.gseg.push_back(g);
                    P->gemm_flops += 2.0 * ld * ob.cols;
                }
                o.s_end = (int64_t)sg.gseg.size();
                sg.gout.push_back(o);
            }
        }
    }
    Stage sr;
    int64_t part_end = 0;
    split_k(sg, QCM_BUF_S2, 0, split_k_segs, sr, part_end);
    for (auto& a : sr.aout) P->axpy_bytes += 8.0 * a.rows * a.cols * (double)(a.t_end - a.t_begin + 1);
    P->scratch[0] = l_end;
    P->scratch[1] = r_end;
    P->scratch[2] = part_end;
    P->stages.push_back(std::move(sx));
    P->stages.push_back(std::move(z));
    P->stages.push_back(std::move(sg));
    if (!sr.aout.empty()) P->stages.push_back(std::move(sr));
    return P;
}

// Gradient of the local energy E = <psi| H_eff psi> (the sigma plan's
// contraction, E = sum over psi blocks of <psi, sigma>) with respect to every
// MPO term scale w: E is linear in each K2 coefficient alpha_k = w_tt a_k, so
//   dE/dw_tt = sum over the K2 terms k of tt of a_k <T[src_k], Y[dst_k]>,
// with Y = dE/dcontr the adjoint of K3: for the K3 segment
// sigma_ob += alpha contr_a op(R), Y_a = alpha psi_ob op(R)^T.  Stages: psi
// right-paired (S0), K1 (T in S1), Y (grouped GEMM into S2, contr's layout),
// then the per-term dots (into S0) and the per-term-scale sums (into OUT).
static qcm_plan* build_grad(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& psi,
                            const std::vector<BM>& L, const std::vector<BM>& R, const MpoV& W, bool herm) {
    auto* P = new qcm_plan();
    P->kind = PK_GRAD;
    const qcm_mpo_t* m = W.m;
    if ((int)L.size() != m->row_dim || (int)R.size() != m->col_dim)
        throw std::runtime_error("boundary aux dimensions do not match the MPO");
    Idx out_left_i = index_product(phys, left_i);
    Idx rib = right_i;
    common_subset(out_left_i, rib);
    PB out_left_pb(phys, left_i, false), in_right_pb(phys, right_i, true);
    Stage z0; z0.kind = ST_ZERO; z0.zbuf = QCM_BUF_S0;
    Stage s0; int64_t rp_end = 0;
    BM rp = plan_reshape_l2r(phys, left_i, right_i, psi, QCM_BUF_KET, QCM_BUF_S0, s0, P, rp_end);
    z0.zlen = rp_end;
    Idx ref;
    for (auto& b : rp.b) ref.d.push_back({b.lc, b.rows});
    Stage s1; int64_t t_end = 0;
    std::vector<BM> T = plan_k1(L, W, herm, rp, QCM_BUF_S0, ref, QCM_BUF_S1, s1, P, t_end);
    std::vector<int> b2list;
    for (int b2 = 0; b2 < m->col_dim; ++b2) b2list.push_back(b2);
    Stage k2; int64_t c_end = 0;
    std::vector<std::pair<int32_t, double>> prov;
    std::vector<BM> C = plan_k2(T, W, b2list, right_i, out_left_i, in_right_pb, out_left_pb, QCM_BUF_S1,
                                QCM_BUF_S2, k2, P, c_end, &prov);
    // Y = dE/dcontr in S2 (blocks no K3 segment reads stay zero)
    Stage zy; zy.kind = ST_ZERO; zy.zbuf = QCM_BUF_S2; zy.zlen = c_end;
    Stage sy; sy.kind = ST_GEMM;
    for (auto& ob : psi.b) {
        if (!(ob.lc == ob.rc)) throw std::runtime_error("psi layout is not block diagonal (left-paired)");
        Q al = ob.lc;
        for (int b2 = 0; b2 < m->col_dim; ++b2) {
            const BM& cb = C[b2];
            size_t it = cb.left_lower_bound(al);
            for (; it < cb.b.size() && cb.b[it].lc == al; ++it) {
                const Blk& a = cb.b[it];
                Q ar = a.rc;
                GemmSeg s;
                s.a_buf = QCM_BUF_KET; s.ta = 0; s.a_off = ob.off; s.lda = ob.rows; s.K = ob.cols;
                if (herm && W.rskip(b2)) {
                    // K3 read R_conj (al, ar) transposed: Y_a = alpha psi_ob R_conj
                    const BM& rs = R[W.rconj(b2)];
                    size_t k = rs.find(al, ar);
                    if (k == rs.b.size()) continue;
                    s.b_buf = QCM_BUF_RIGHT; s.tb = 0; s.b_off = rs.b[k].off; s.ldb = rs.b[k].rows;
                    s.alpha = W.conj_scale(ar.s, al.s, W.rspin(b2), W.rphase(W.rconj(b2)));
                    if (rs.b[k].cols != a.cols || rs.b[k].rows != ob.cols)
                        throw std::runtime_error("gradient: K3 dimension mismatch (adjoint)");
                } else {
                    // K3 read R (ar, al): Y_a = psi_ob R^T
                    const BM& rs = R[b2];
                    size_t k = rs.find(ar, al);
                    if (k == rs.b.size()) continue;
                    s.b_buf = QCM_BUF_RIGHT; s.tb = 1; s.b_off = rs.b[k].off; s.ldb = rs.b[k].rows;
                    s.alpha = 1.0;
                    if (rs.b[k].rows != a.cols || rs.b[k].cols != ob.cols)
                        throw std::runtime_error("gradient: K3 dimension mismatch");
                }
                if (a.rows != ob.rows) throw std::runtime_error("gradient: K3 row mismatch");
                GemmOut o;
                o.c_buf = QCM_BUF_S2; o.c_off = a.off; o.ldc = a.rows; o.M = a.rows; o.N = a.cols;
                o.s_begin = (int64_t)sy.gseg.size();
                sy.gseg.push_back(s);
                o.s_end = (int64_t)sy.gseg.size();
                sy.gout.push_back(o);
                P->gemm_flops += 2.0 * a.rows * a.cols * ob.cols;
            }
        }
    }
    // the per-term dots of K2's tables against Y, and the sums per MPO term scale
    Stage sd; sd.kind = ST_DOT;
    sd.aout = std::move(k2.aout);
    sd.aterm = std::move(k2.aterm);
    sd.dot_w.resize(prov.size());
    sd.dot_tt.resize(prov.size());
    for (size_t k = 0; k < prov.size(); ++k) {
        sd.dot_tt[k] = prov[k].first;
        sd.dot_w[k] = prov[k].second;
    }
    // the output tiles already point into S2, where Y has contr's layout
    for (const AxpyOut& o : sd.aout) P->axpy_flops += 2.0 * o.rows * o.cols * (double)(o.t_end - o.t_begin);
    sd.dot_buf = QCM_BUF_S0;
    sd.n_tt = m->term_ptr[m->col_ptr[m->col_dim]];
    P->out_elems = sd.n_tt;
    P->scratch[0] = std::max(rp_end, (int64_t)sd.aterm.size());
    P->scratch[1] = t_end;
    P->scratch[2] = c_end;
    P->stages.push_back(std::move(z0));
    P->stages.push_back(std::move(s0));
    P->stages.push_back(std::move(s1));
    P->stages.push_back(std::move(zy));
    P->stages.push_back(std::move(sy));
    P->stages.push_back(std::move(sd));
    return P;
}

// tensor_mpo: the plan stops after the operator application and writes it to
// OUT as a boundary with one block matrix per right MPO bond -- every bond,
// as left_boundary_tensor_mpo computes them (move_boundary.hpp:66-97): the
// boundary x MPS product is trimmed to the ket's left index and the output
// rows are not restricted to the right index.
static qcm_plan* build_bleft(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& mps,
                             const std::vector<BM>& L, const MpoV& W, bool herm, bool tensor_mpo = false) {
    auto* P = new qcm_plan();
    P->kind = PK_BLEFT;
    const qcm_mpo_t* m = W.m;
    if ((int)L.size() != m->row_dim) throw std::runtime_error("left boundary aux dimension does not match the MPO");
    Idx out_left_i = index_product(phys, left_i);
    Idx rib = right_i;
    if (!tensor_mpo) common_subset(out_left_i, rib);
    PB out_left_pb(phys, left_i, false), in_right_pb(phys, right_i, true);
    Stage z0; z0.kind = ST_ZERO; z0.zbuf = QCM_BUF_S0;
    Stage s0; int64_t rp_end = 0;
    BM rp = plan_reshape_l2r(phys, left_i, right_i, mps, QCM_BUF_KET, QCM_BUF_S0, s0, P, rp_end);
    z0.zlen = rp_end;
    Idx ref;
    if (tensor_mpo) ref = left_i;
    else for (auto& b : rp.b) ref.d.push_back({b.lc, b.rows});
    Stage s1; int64_t t_end = 0;
    std::vector<BM> T = plan_k1(L, W, herm, rp, QCM_BUF_S0, ref, QCM_BUF_S1, s1, P, t_end, true, kTAlign);
    std::vector<int> b2list;
    for (int b2 = 0; b2 < m->col_dim; ++b2)
        if (tensor_mpo || !(herm && W.rskip(b2))) b2list.push_back(b2);
    Stage s2; int64_t c_end = 0;
    const int32_t c_buf = tensor_mpo ? QCM_BUF_OUT : QCM_BUF_S2;
    std::vector<BM> C = plan_k2(T, W, b2list, right_i, out_left_i, in_right_pb, out_left_pb, QCM_BUF_S1,
                                c_buf, s2, P, c_end, nullptr, W.abelian());
    Stage z2; z2.kind = ST_ZERO; z2.zbuf = c_buf; z2.zlen = c_end;
    if (tensor_mpo) {
        // C already carries its offsets in OUT, bond after bond
        P->out_blk_ptr.assign(1, 0);
        for (auto& bm : C) {
            for (auto& b : bm.b) P->out_blocks.push_back(b);
            P->out_blk_ptr.push_back((int32_t)P->out_blocks.size());
        }
        P->out_elems = c_end;
        P->scratch[0] = rp_end;
        P->scratch[1] = t_end;
        build_image_tables(s1, s1.img);
        axpy_components(s2, s2.comp_root);
        build_dense_groups(s2, 64, s2.img, s2.heavy);
        P->image_bytes = std::max(s1.img.bytes, s2.img.bytes);
        P->stages.push_back(std::move(z0));
        P->stages.push_back(std::move(s0));
        P->stages.push_back(std::move(s1));
        P->stages.push_back(std::move(z2));
        P->stages.push_back(std::move(s2));
        return P;
    }
    // ret[b2] = SU2::gemm(transpose(contr[b2]), bra_lp, right_spin(b2))
    std::vector<BM> out(m->col_dim);
    struct Job { int b2; Q lc, rc; int64_t a_off, a_rows, a_cols; size_t bk; };
    std::vector<Job> jobs;
    for (int b2 : b2list) {
        // transposed blocks in sorted order
        std::vector<Blk> At;
        for (auto& x : C[b2].b) { Blk t = x; std::swap(t.lc, t.rc); At.push_back(t); }
        std::stable_sort(At.begin(), At.end(), [](const Blk& p, const Blk& q) {
            return p.lc > q.lc || (p.lc == q.lc && p.rc > q.rc);
        });
        for (auto& a : At) {
            Q ar = a.rc;  // out_l
            size_t it = mps.left_lower_bound(ar);
            for (; it < mps.b.size() && mps.b[it].lc == ar; ++it) {
                if (!W.allowed(a.lc.s, W.rspin(b2), mps.b[it].rc.s)) continue;
                Blk nb;
                nb.lc = a.lc;
                nb.rc = mps.b[it].rc;
                nb.rows = a.cols;       // transposed: rows of A^T = cols of contr block
                nb.cols = mps.b[it].cols;
                if (out[b2].find(nb.lc, nb.rc) != out[b2].b.size()) throw std::runtime_error("duplicate L block");
                out[b2].insert(nb);
                jobs.push_back({b2, nb.lc, nb.rc, a.off, a.rows, a.cols, it});
            }
        }
    }
    finalize_boundary_layout(P, out);
    Stage s3; s3.kind = ST_GEMM;
    for (auto& j : jobs) {
        const Blk& c = out[j.b2].b[out[j.b2].find(j.lc, j.rc)];
        const Blk& bb = mps.b[j.bk];
        GemmOut o;
        o.c_buf = QCM_BUF_OUT; o.c_off = c.off; o.ldc = c.rows; o.M = c.rows; o.N = c.cols;
        o.s_begin = (int64_t)s3.gseg.size();
        GemmSeg s;
        s.a_buf = QCM_BUF_S2; s.ta = 1; s.a_off = j.a_off; s.lda = j.a_rows;
        s.b_buf = QCM_BUF_KET; s.tb = 0; s.b_off = bb.off; s.ldb = bb.rows;
        s.K = j.a_rows; s.alpha = 1.0;
        if (bb.rows != j.a_rows) throw std::runtime_error("left step inner dimension mismatch");
        s3.gseg.push_back(s);
        o.s_end = (int64_t)s3.gseg.size();
        s3.gout.push_back(o);
        P->gemm_flops += 2.0 * c.rows * c.cols * j.a_rows;
    }
    P->scratch[0] = rp_end;
    P->scratch[1] = t_end;
    P->scratch[2] = c_end;
    build_image_tables(s1, s1.img);
    build_image_tables(s3, s3.img);
    axpy_components(s2, s2.comp_root);
    build_dense_groups(s2, 64, s2.img, s2.heavy);
    P->image_bytes = std::max(std::max(s1.img.bytes, s3.img.bytes), s2.img.bytes);
    P->stages.push_back(std::move(z0));
    P->stages.push_back(std::move(s0));
    P->stages.push_back(std::move(s1));
    P->stages.push_back(std::move(z2));
    P->stages.push_back(std::move(s2));
    P->stages.push_back(std::move(s3));
    return P;
}

// tensor_mpo: as for build_bleft, the plan ends after the operator application
// and writes every left MPO bond's block matrix to OUT, as
// right_boundary_tensor_mpo computes them (move_boundary.hpp:99-126): the
// MPS x boundary product is trimmed to the ket's *left* index (the index
// MPSBoundaryProduct's three-argument constructor passes,
// boundary_times_mps.hpp:258-261) and the output columns are not restricted
// to the left index.
static qcm_plan* build_bright(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& mps,
                              const std::vector<BM>& R, const MpoV& W, bool herm, bool tensor_mpo = false) {
    auto* P = new qcm_plan();
    P->kind = PK_BRIGHT;
    const qcm_mpo_t* m = W.m;
    if ((int)R.size() != m->col_dim) throw std::runtime_error("right boundary aux dimension does not match the MPO");
    Idx out_right_i = index_product(adjoin(phys), right_i);
    Idx bli = left_i;
    if (!tensor_mpo) common_subset(out_right_i, bli);
    PB in_left_pb(phys, left_i, false), out_right_pb(phys, right_i, true);
    Idx ref;  // bra (left-paired) right basis
    if (tensor_mpo) ref = left_i;
    else for (auto& b : mps.b) ref.d.push_back({b.rc, b.cols});
    // t[b2] = mps_lp . R'[b2]  (gemm_trim_right)
    std::vector<BM> t(m->col_dim);
    struct Job { int b2; Q lc, rc; size_t ak; int64_t b_off, ldb; int tb; double sc; int64_t N; };
    std::vector<Job> jobs;
    for (int b2 = 0; b2 < m->col_dim; ++b2) {
        bool use_conj = herm && W.rskip(b2);
        std::vector<Blk> Bb;
        std::vector<double> sc;
        std::vector<int> tbv;
        if (use_conj) {
            const BM& src = R[W.rconj(b2)];
            for (auto& x : src.b) { Blk tt = x; std::swap(tt.lc, tt.rc); Bb.push_back(tt); }
        } else {
            Bb = R[b2].b;
        }
        std::vector<size_t> order(Bb.size());
        for (size_t i = 0; i < order.size(); ++i) order[i] = i;
        std::stable_sort(order.begin(), order.end(), [&](size_t p, size_t q) {
            return Bb[p].lc > Bb[q].lc || (Bb[p].lc == Bb[q].lc && Bb[p].rc > Bb[q].rc);
        });
        BM Bs;
        for (size_t i : order) Bs.b.push_back(Bb[i]);
        for (size_t ak = 0; ak < mps.b.size(); ++ak) {
            const Blk& a = mps.b[ak];
            size_t it = Bs.left_lower_bound(a.rc);
            for (; it < Bs.b.size() && Bs.b[it].lc == a.rc; ++it) {
                const Blk& bb = Bs.b[it];
                if (!ref.has(bb.rc)) continue;
                Blk nb;
                nb.lc = a.lc;
                nb.rc = bb.rc;
                nb.rows = a.rows;
                // conj: stored block is (rc, lc) of R[conj] with rows = its own rows -> N = stored rows
                nb.cols = use_conj ? bb.rows : bb.cols;
                if (t[b2].find(nb.lc, nb.rc) != t[b2].b.size()) throw std::runtime_error("duplicate t block");
                t[b2].insert(nb);
                double s = use_conj ? W.conj_scale(bb.lc.s, bb.rc.s, W.rspin(b2), W.rphase(W.rconj(b2))) : 1.0;
                jobs.push_back({b2, nb.lc, nb.rc, ak, bb.off, bb.rows, use_conj ? 1 : 0, s, nb.cols});
            }
        }
    }
    int64_t t_end = 0;
    for (auto& x : t) t_end = x.assign_offsets(t_end);
    Stage s1; s1.kind = ST_GEMM;
    for (auto& j : jobs) {
        const Blk& c = t[j.b2].b[t[j.b2].find(j.lc, j.rc)];
        const Blk& a = mps.b[j.ak];
        GemmOut o;
        o.c_buf = QCM_BUF_S1; o.c_off = c.off; o.ldc = c.rows; o.M = c.rows; o.N = c.cols;
        o.s_begin = (int64_t)s1.gseg.size();
        GemmSeg s;
        s.a_buf = QCM_BUF_KET; s.ta = 0; s.a_off = a.off; s.lda = a.rows;
        s.b_buf = QCM_BUF_RIGHT; s.tb = j.tb; s.b_off = j.b_off; s.ldb = j.ldb;
        s.K = a.cols; s.alpha = j.sc;
        s1.gseg.push_back(s);
        o.s_end = (int64_t)s1.gseg.size();
        s1.gout.push_back(o);
        P->gemm_flops += 2.0 * c.rows * c.cols * a.cols;
    }
    // rbtm tasks into buf[b1](out_l, out_r), one host task per b1: its terms in loop
    // order, each keyed by its tile (out_l, out_r, column offset), then stably ordered
    // by tile as the reference's block order (both charges descending, offsets
    // ascending); the tiles go out in b1 order
    struct RTerm { Q out_l, out_r; int64_t col, rows, cols; AxpyTerm t; };
    struct RowOut { std::vector<RTerm> terms; std::vector<uint32_t> order; double flops = 0.0; };
    std::vector<RowOut> rows_out(m->row_dim);
    std::vector<BM> buf(m->row_dim);
    MpoV const& Wv = W;
    parallel_for((size_t)m->row_dim, [&](size_t b1s) {
        const int b1 = (int)b1s;
        if (herm && !tensor_mpo && Wv.lskip(b1)) return;
        RowOut& ro = rows_out[b1];
        int a = Wv.lspin(b1);
        for (size_t r = 0; r < Wv.row_b2[b1].size(); ++r) {
            int b2 = Wv.row_b2[b1][r];
            int e = Wv.row_elem[b1][r];
            int ap = Wv.rspin(b2);
            for (int tt = m->term_ptr[e]; tt < m->term_ptr[e + 1]; ++tt) {
                int op = m->term_op[tt];
                double scale = m->term_scale[tt];
                int k = m->op_spin[op];
                for (auto& tb : t[b2].b) {
                    Q lc = tb.lc, rc = tb.rc, mc = tb.lc;
                    for (int wb = m->op_blk_ptr[op]; wb < m->op_blk_ptr[op + 1]; ++wb) {
                        Q pin(m->blk_q[4 * wb], m->blk_q[4 * wb + 1]), pout(m->blk_q[4 * wb + 2], m->blk_q[4 * wb + 3]);
                        Q out_l = fuse(lc, neg(pin));
                        size_t lb = left_i.position(out_l);
                        if (lb == left_i.size()) continue;
                        Q out_r = fuse(rc, neg(pout));
                        if (!Wv.allowed(out_l.s, a, out_r.s)) continue;
                        if (!out_right_i.has(out_r)) continue;
                        int64_t l_size = left_i.d[lb].second;
                        int i = out_r.s, ip = rc.s, j = out_l.s, jp = mc.s;
                        double cpl[4];
                        Wv.coupling(j, jp, a, k, ap, i, ip, scale, cpl);
                        int64_t ilo = in_left_pb(pin, out_l), oro = out_right_pb(pout, rc);
                        int64_t r_size = tb.cols;
                        if (buf[b1].find(out_l, out_r) == buf[b1].b.size()) {
                            Blk nb;
                            nb.lc = out_l; nb.rc = out_r; nb.rows = l_size; nb.cols = out_right_i.size_of(out_r);
                            buf[b1].insert(nb);
                        }
                        for (int en = m->blk_ent_ptr[wb]; en < m->blk_ent_ptr[wb + 1]; ++en) {
                            int ss1 = m->ent[4 * en], ss2 = m->ent[4 * en + 1];
                            double alfa = m->ent_coeff[en] * cpl[spin_case(m->ent[4 * en + 2], m->ent[4 * en + 3])];
                            if (alfa == 0.0) continue;
                            ro.terms.push_back({out_l, out_r, oro + (int64_t)ss2 * r_size, l_size, r_size,
                                                {QCM_BUF_S1, tb.off + ilo + (int64_t)ss1 * l_size, tb.rows, alfa}});
                            ro.flops += 2.0 * l_size * r_size;
                        }
                    }
                }
            }
        }
        if (Wv.abelian()) {
            // rbtm_kernel_allocate (ct/abelian/apply_op.hpp:140-187): for every (b2, operator)
            // of the row with a non-empty t[b2], one block per left sector at the constant
            // charge shifts, whether or not a term writes it (zero, but part of the layout)
            for (size_t r = 0; r < Wv.row_b2[b1].size(); ++r) {
                const int b2 = Wv.row_b2[b1][r], e = Wv.row_elem[b1][r];
                if (t[b2].b.empty()) continue;
                const Q t_delta = fuse(t[b2].b[0].rc, neg(t[b2].b[0].lc));
                for (int tt = m->term_ptr[e]; tt < m->term_ptr[e + 1]; ++tt) {
                    const int op = m->term_op[tt];
                    if (m->op_blk_ptr[op] == m->op_blk_ptr[op + 1]) continue;
                    const int w0 = m->op_blk_ptr[op];
                    const Q op_delta = fuse(Q(m->blk_q[4 * w0 + 2], m->blk_q[4 * w0 + 3]),
                                            neg(Q(m->blk_q[4 * w0], m->blk_q[4 * w0 + 1])));
                    const Q total = fuse(op_delta, neg(t_delta));
                    for (auto& ls : left_i.d) {
                        const Q out_r = fuse(ls.first, neg(total));
                        if (!out_right_i.has(out_r) || buf[b1].find(ls.first, out_r) != buf[b1].b.size()) continue;
                        Blk nb;
                        nb.lc = ls.first; nb.rc = out_r; nb.rows = ls.second; nb.cols = out_right_i.size_of(out_r);
                        buf[b1].insert(nb);
                    }
                }
            }
        }
        ro.order.resize(ro.terms.size());
        std::iota(ro.order.begin(), ro.order.end(), 0u);
        const std::vector<RTerm>& ts = ro.terms;
        std::stable_sort(ro.order.begin(), ro.order.end(), [&](uint32_t x, uint32_t y) {
            const RTerm &u = ts[x], &v = ts[y];
            if (!(u.out_l == v.out_l)) return u.out_l > v.out_l;
            if (!(u.out_r == v.out_r)) return u.out_r > v.out_r;
            return u.col < v.col;
        });
    });
    int64_t b_end = 0;
    for (auto& x : buf) b_end = x.assign_offsets(b_end);
    const int32_t buf_slot = tensor_mpo ? QCM_BUF_OUT : QCM_BUF_S2;
    Stage z2; z2.kind = ST_ZERO; z2.zbuf = buf_slot; z2.zlen = b_end;
    Stage s2; s2.kind = ST_AXPY;
    {
        size_t nterms = 0;
        for (const RowOut& ro : rows_out) nterms += ro.terms.size();
        s2.aterm.reserve(nterms);
    }
    for (int b1 = 0; b1 < m->row_dim; ++b1) {
        const RowOut& ro = rows_out[b1];
        P->axpy_flops += ro.flops;
        for (size_t g0 = 0; g0 < ro.order.size();) {
            const RTerm& k0 = ro.terms[ro.order[g0]];
            size_t g1 = g0 + 1;
            while (g1 < ro.order.size()) {
                const RTerm& k1 = ro.terms[ro.order[g1]];
                if (!(k1.out_l == k0.out_l) || !(k1.out_r == k0.out_r) || k1.col != k0.col) break;
                ++g1;
            }
            const Blk& d = buf[b1].b[buf[b1].find(k0.out_l, k0.out_r)];
            const RTerm& last = ro.terms[ro.order[g1 - 1]];
            AxpyOut o;
            o.dst_buf = buf_slot;
            o.dst_off = d.off + k0.col * d.rows;
            o.ldd = d.rows;
            o.rows = last.rows;
            o.cols = last.cols;
            o.t_begin = (int64_t)s2.aterm.size();
            for (size_t g = g0; g < g1; ++g) s2.aterm.push_back(ro.terms[ro.order[g]].t);
            o.t_end = (int64_t)s2.aterm.size();
            s2.aout.push_back(o);
            P->axpy_bytes += 8.0 * o.rows * o.cols * (double)(g1 - g0 + 1);
            g0 = g1;
        }
    }
    if (tensor_mpo) {
        P->out_blk_ptr.assign(1, 0);
        for (auto& bm : buf) {
            for (auto& b : bm.b) P->out_blocks.push_back(b);
            P->out_blk_ptr.push_back((int32_t)P->out_blocks.size());
        }
        P->out_elems = b_end;
        P->scratch[1] = t_end;
        build_image_tables(s1, s1.img);
        axpy_components(s2, s2.comp_root);
        build_dense_groups(s2, 64, s2.img, s2.heavy);
        P->image_bytes = std::max(s1.img.bytes, s2.img.bytes);
        P->stages.push_back(std::move(s1));
        P->stages.push_back(std::move(z2));
        P->stages.push_back(std::move(s2));
        return P;
    }
    // bra right-paired copy for the final product
    Stage z0; z0.kind = ST_ZERO; z0.zbuf = QCM_BUF_S0;
    Stage s0; int64_t rp_end = 0;
    BM rp = plan_reshape_l2r(phys, left_i, right_i, mps, QCM_BUF_KET, QCM_BUF_S0, s0, P, rp_end);
    z0.zlen = rp_end;
    // ret[b1] = SU2::gemm(buf[b1], transpose(bra_rp), left_spin(b1))
    std::vector<BM> out(m->row_dim);
    struct J3 { int b1; Q lc, rc; int64_t a_off, a_rows, a_cols; size_t bk; };
    std::vector<J3> j3;
    for (int b1 = 0; b1 < m->row_dim; ++b1) {
        for (auto& a : buf[b1].b) {
            Q ar = a.rc;
            size_t k = rp.find(ar, ar);
            if (k == rp.b.size()) continue;
            if (!Wv.allowed(a.lc.s, Wv.lspin(b1), ar.s)) continue;
            Blk nb;
            nb.lc = a.lc; nb.rc = ar; nb.rows = a.rows; nb.cols = rp.b[k].rows;
            out[b1].insert(nb);
            if (rp.b[k].cols != a.cols) throw std::runtime_error("right step inner dimension mismatch");
            j3.push_back({b1, nb.lc, nb.rc, a.off, a.rows, a.cols, k});
        }
    }
    finalize_boundary_layout(P, out);
    Stage s3; s3.kind = ST_GEMM;
    for (auto& j : j3) {
        const Blk& c = out[j.b1].b[out[j.b1].find(j.lc, j.rc)];
        const Blk& bb = rp.b[j.bk];
        GemmOut o;
        o.c_buf = QCM_BUF_OUT; o.c_off = c.off; o.ldc = c.rows; o.M = c.rows; o.N = c.cols;
        o.s_begin = (int64_t)s3.gseg.size();
        GemmSeg s;
        s.a_buf = QCM_BUF_S2; s.ta = 0; s.a_off = j.a_off; s.lda = j.a_rows;
        s.b_buf = QCM_BUF_S0; s.tb = 1; s.b_off = bb.off; s.ldb = bb.rows;
        s.K = j.a_cols; s.alpha = 1.0;
        s3.gseg.push_back(s);
        o.s_end = (int64_t)s3.gseg.size();
        s3.gout.push_back(o);
        P->gemm_flops += 2.0 * c.rows * c.cols * j.a_cols;
    }
    P->scratch[0] = rp_end;
    P->scratch[1] = t_end;
    P->scratch[2] = b_end;
    build_image_tables(s1, s1.img);
    build_image_tables(s3, s3.img);
    axpy_components(s2, s2.comp_root);
    build_dense_groups(s2, 64, s2.img, s2.heavy);
    P->image_bytes = std::max(std::max(s1.img.bytes, s3.img.bytes), s2.img.bytes);
    P->stages.push_back(std::move(s1));
    P->stages.push_back(std::move(z2));
    P->stages.push_back(std::move(s2));
    P->stages.push_back(std::move(z0));
    P->stages.push_back(std::move(s0));
    P->stages.push_back(std::move(s3));
    return P;
}

// Image tables of one GEMM stage.  Each output is computed as a D tile of
// the MMA with the larger of (M, N) on the 128-row MMA side: when N > M the
// stage's C = op(A) op(B) is computed as C^T = op(B)^T op(A)^T (less padding;
// the other choice, with coalesced column stores, was measured slower for K1).
// Panels that several segments read with the same orientation share one image.
void build_image_tables(const Stage& st, ImgTables& t, int n_tile_max, bool a_resident) {
    t = ImgTables();
    struct Key {
        int32_t buf, ld, R, K, kc;
        int64_t off;
        bool operator==(const Key& o) const {
            return buf == o.buf && ld == o.ld && R == o.R && K == o.K && kc == o.kc && off == o.off;
        }
    };
    struct KeyHash {
        size_t operator()(const Key& k) const {
            uint64_t h = (uint64_t)k.off * 0x9E3779B97F4A7C15ull;
            h ^= ((uint64_t)k.buf << 48) ^ ((uint64_t)k.kc << 47) ^ ((uint64_t)k.R << 24) ^ (uint64_t)k.K;
            h ^= (uint64_t)k.ld * 0xC2B2AE3D27D4EB4Full;
            return (size_t)(h ^ (h >> 29));
        }
    };
    std::unordered_map<Key, int32_t, KeyHash> ids;
    // a panel gets an image (and image-builder work) the first time a segment reads it from one
    auto give_image = [&](int32_t id) {
        ImgPanel& p = t.panels[id];
        if (p.img_off >= 0) return;
        p.img_off = t.bytes;
        const int64_t kc = (p.K + 31) / 32;
        t.bytes += kc * 3 * (int64_t)p.G * 512;
        for (int64_t c = 0; c < kc; ++c) { t.build.push_back(id); t.build.push_back((int32_t)c); }
    };
    auto panel = [&](int32_t buf, int64_t off, int64_t ld, int kcontig, int64_t R, int64_t K, bool image) -> int32_t {
        Key k{buf, (int32_t)ld, (int32_t)R, (int32_t)K, kcontig, off};
        auto it = ids.find(k);
        if (it != ids.end()) {
            if (image) give_image(it->second);
            return it->second;
        }
        ImgPanel p;
        p.src_off = off;
        p.src_buf = buf;
        p.ld = (int32_t)ld;
        p.R = (int32_t)R;
        p.K = (int32_t)K;
        p.kcontig = kcontig;
        p.G = (int32_t)((R + 7) / 8);
        p.img_off = -1;
        const int32_t id = (int32_t)t.panels.size();
        t.panels.push_back(p);
        ids.emplace(k, id);
        if (image) give_image(id);
        return id;
    };
    for (const GemmOut& o : st.gout) {
        if (o.M > 0x7fffffff || o.N > 0x7fffffff || o.ldc > 0x7fffffff)
            throw std::runtime_error("image executor: block too large");
        const bool tr = o.N > o.M;
        ImgOut io;
        io.c_off = o.c_off;
        io.c_buf = o.c_buf;
        io.si = tr ? o.ldc : 1;
        io.sj = tr ? 1 : o.ldc;
        io.mrows = (int32_t)(tr ? o.N : o.M);
        io.ncols = (int32_t)(tr ? o.M : o.N);
        io.ctab = 0;
        io.mode = 0;
        io.rows = 0;
        // transposed tiles of a padded output store 4 contiguous rows per vector
        io.pad = tr && o.vec_store ? 1 : 0;
        const int32_t oid = (int32_t)t.outs.size();
        t.outs.push_back(io);
        const int32_t s_begin = (int32_t)t.segs.size();
        for (int64_t si = o.s_begin; si < o.s_end; ++si) {
            const GemmSeg& g = st.gseg[si];
            if (g.K <= 0) continue;
            if (g.lda > 0x7fffffff || g.ldb > 0x7fffffff || g.K > 0x7fffffff)
                throw std::runtime_error("image executor: block too large");
            // op(A): rows m, element (m,k) at ta ? k + m*lda : m + k*lda
            // op(B)^T: rows n, element (n,k) = op(B)(k,n) at tb ? n + k*ldb : k + n*ldb
            const int32_t pa = panel(g.a_buf, g.a_off, g.lda, g.ta ? 1 : 0, o.M, g.K, true);
            const int32_t pb = panel(g.b_buf, g.b_off, g.ldb, g.tb ? 0 : 1, o.N, g.K, true);
            const int32_t ia = tr ? pb : pa, ib = tr ? pa : pb;
            const ImgPanel& A = t.panels[ia];
            const ImgPanel& B = t.panels[ib];
            ImgSeg s;
            s.a_img = A.img_off;
            s.b_img = B.img_off;
            s.a_G = A.G;
            s.b_G = B.G;
            s.kc = (int32_t)((g.K + 31) / 32);
            s.alpha = (float)g.alpha;
            s.flags = 0;
            s.a_panel = ia;
            s.a_c0 = 0;
            s.pad = 0;
            t.segs.push_back(s);
        }
        const int32_t s_end = (int32_t)t.segs.size();
        // N tiles of balanced width (multiples of 16, at most n_tile_max): e.g. 160 = 80 + 80
        const int32_t nnt = (io.ncols + n_tile_max - 1) / n_tile_max;
        const int32_t per = ((io.ncols + nnt - 1) / nnt + 15) / 16 * 16;
        for (int32_t m0 = 0; m0 < io.mrows; m0 += 128)
            for (int32_t n0 = 0; n0 < io.ncols; n0 += per) {
                ImgUnit u;
                u.out = oid;
                u.m0 = m0;
                u.n0 = n0;
                u.nt = std::min(per, (io.ncols - n0 + 15) / 16 * 16);
                u.s_begin = s_begin;
                u.s_end = s_end;
                t.units.push_back(u);
            }
    }
    if (t.build.size() / 2 > 0x7fffffffULL || t.units.size() > 0x7fffffffULL || t.segs.size() > 0x7fffffffULL)
        throw std::runtime_error("image executor: tables too large");
    // A-resident mode when every tile is a single short segment (K1: each T tile is one
    // block product; the same psi tile is the A operand of hundreds of products)
    bool ares = a_resident && !t.units.empty();
    for (const ImgUnit& u : t.units)
        ares = ares && u.s_end - u.s_begin == 1 && t.segs[u.s_begin].kc <= IMG_ARES_MAX;
    if (ares) {
        std::stable_sort(t.units.begin(), t.units.end(), [&](const ImgUnit& x, const ImgUnit& y) {
            const int64_t ax = t.segs[x.s_begin].a_img, ay = t.segs[y.s_begin].a_img;
            return ax != ay ? ax < ay : x.m0 < y.m0;
        });
        t.ares = true;
        t.cost.assign(t.units.size() + 1, 0);
        for (size_t i = 0; i < t.units.size(); ++i)
            t.cost[i + 1] = t.cost[i] + (int64_t)t.segs[t.units[i].s_begin].kc * (t.units[i].nt + 32) + 64;
    }
}

// Round-to-nearest-even FP32 -> BF16 (finite inputs) and back.
static uint16_t bf16_rne(float x) {
    uint32_t u;
    std::memcpy(&u, &x, 4);
    u += 0x7FFFu + ((u >> 16) & 1u);
    return (uint16_t)(u >> 16);
}
static float bf16_to_float(uint16_t h) {
    const uint32_t u = (uint32_t)h << 16;
    float x;
    std::memcpy(&x, &u, 4);
    return x;
}

int64_t tile_pitch(const Stage& st, const AxpyOut& a) {
    if (a.t_end == a.t_begin || a.cols <= 1) return a.rows;
    const int64_t p = st.aterm[a.t_begin].lds;
    if (p < a.rows || p > (a.rows + 3) / 4 * 4) return -1;
    for (int64_t t = a.t_begin; t < a.t_end; ++t)
        if (st.aterm[t].lds != p) return -1;
    return p;
}

bool axpy_components(const Stage& st, std::vector<int32_t>& root) {
    const size_t nO = st.aout.size();
    const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    auto run = [&](const std::function<void(unsigned)>& f) {
        std::vector<std::thread> pool;
        for (unsigned t = 1; t < nt; ++t) pool.emplace_back(f, t);
        f(0);
        for (auto& th : pool) th.join();
    };
    std::atomic<bool> contiguous{true};
    run([&](unsigned t) {
        for (size_t i = t; i < nO && contiguous.load(std::memory_order_relaxed); i += nt) {
            if (tile_pitch(st, st.aout[i]) < 0) { contiguous = false; break; }
        }
    });
    if (!contiguous) return false;
    // lock-free union-find: a root is only ever linked under a smaller root (CAS on
    // the root's own entry), so every component ends with its smallest output as root
    std::vector<std::atomic<int32_t>> parent(nO);
    for (size_t i = 0; i < nO; ++i) parent[i].store((int32_t)i, std::memory_order_relaxed);
    auto find = [&](int32_t x) {
        for (;;) {
            const int32_t p = parent[x].load(std::memory_order_relaxed);
            if (p == x) return x;
            x = p;
        }
    };
    auto unite = [&](int32_t a, int32_t b) {
        for (;;) {
            a = find(a);
            b = find(b);
            if (a == b) return;
            if (a > b) std::swap(a, b);
            int32_t expect = b;
            if (parent[b].compare_exchange_strong(expect, a)) return;
        }
    };
    // every thread owns the source keys of one hash class: it keeps their first output
    // in a private open-addressing table and unites later readers with it.  The terms
    // are read once: each thread buckets the (key, output) pairs of its share of the
    // outputs by class, then the owner of a class walks the buckets in output order.
    // (The components, and so every root, do not depend on the walk order.)
    auto mix = [](int64_t key) { return (uint64_t)key * 0x9E3779B97F4A7C15ull; };
    std::vector<std::vector<std::vector<std::pair<int64_t, int32_t>>>> bucket(
        nt, std::vector<std::vector<std::pair<int64_t, int32_t>>>(nt));
    run([&](unsigned t) {
        const size_t i0 = nO * t / nt, i1 = nO * (t + 1) / nt;
        std::vector<size_t> cnt(nt, 0);
        for (size_t i = i0; i < i1; ++i) {
            const AxpyOut& a = st.aout[i];
            for (int64_t k = a.t_begin; k < a.t_end; ++k) {
                const int64_t key = ((int64_t)st.aterm[k].src_buf << 56) ^ st.aterm[k].src_off;
                ++cnt[(mix(key) >> 58) % nt];
            }
        }
        for (unsigned c = 0; c < nt; ++c) bucket[t][c].reserve(cnt[c]);
        for (size_t i = i0; i < i1; ++i) {
            const AxpyOut& a = st.aout[i];
            for (int64_t k = a.t_begin; k < a.t_end; ++k) {
                const int64_t key = ((int64_t)st.aterm[k].src_buf << 56) ^ st.aterm[k].src_off;
                bucket[t][(mix(key) >> 58) % nt].push_back({key, (int32_t)i});
            }
        }
    });
    run([&](unsigned t) {
        std::vector<int64_t> keys(1u << 12, -1);
        std::vector<int32_t> vals(1u << 12, 0);
        size_t used = 0;
        auto slot = [&](int64_t key) {
            const size_t mask = keys.size() - 1;
            size_t h = (size_t)(mix(key) >> 24) & mask;
            while (keys[h] != -1 && keys[h] != key) h = (h + 1) & mask;
            return h;
        };
        for (unsigned src = 0; src < nt; ++src)
            for (const auto& kv : bucket[src][t]) {
                const int64_t key = kv.first;
                const int32_t i = kv.second;
                size_t h = slot(key);
                if (keys[h] == -1) {
                    keys[h] = key;
                    vals[h] = (int32_t)i;
                    if (2 * ++used > keys.size()) {  // grow and rehash
                        std::vector<int64_t> ok;
                        std::vector<int32_t> ov;
                        ok.swap(keys);
                        ov.swap(vals);
                        keys.assign(ok.size() * 2, -1);
                        vals.assign(ok.size() * 2, 0);
                        for (size_t q = 0; q < ok.size(); ++q)
                            if (ok[q] != -1) {
                                const size_t g = slot(ok[q]);
                                keys[g] = ok[q];
                                vals[g] = ov[q];
                            }
                    }
                } else if (vals[h] != i) {
                    unite(i, vals[h]);
                }
            }
        for (unsigned src = 0; src < nt; ++src) std::vector<std::pair<int64_t, int32_t>>().swap(bucket[src][t]);
    });
    root.resize(nO);
    for (size_t i = 0; i < nO; ++i) root[i] = find((int32_t)i);
    return true;
}

void build_dense_groups(const Stage& st, int64_t min_terms, ImgTables& t, std::vector<char>& heavy) {
    t = ImgTables();
    const size_t nO = st.aout.size();
    heavy.assign(nO, 0);
    if (nO == 0) return;
    // connected components of the output/source graph
    std::vector<int32_t> rootv;
    const std::vector<int32_t>* roots = &st.comp_root;
    if (st.comp_root.size() != nO) {
        if (!axpy_components(st, rootv)) return;  // sources must be contiguous tiles
        roots = &rootv;
    }
    auto find = [&](int32_t x) { return (*roots)[x]; };
    // candidate groups: (component, rows, cols, dst_buf, src_buf, pitch) over heavy outputs;
    // a tile is its sources' pitch x cols run, of which the rows < rows are stored
    std::map<std::tuple<int32_t, int64_t, int64_t, int32_t, int32_t, int64_t>, std::vector<int32_t>> groups;
    for (size_t i = 0; i < nO; ++i) {
        const AxpyOut& a = st.aout[i];
        if (a.t_end - a.t_begin < min_terms || a.rows * a.cols <= 0) continue;
        const int32_t sb = st.aterm[a.t_begin].src_buf;
        bool uniform = true;
        for (int64_t k = a.t_begin; k < a.t_end; ++k) uniform &= st.aterm[k].src_buf == sb;
        if (!uniform) continue;
        if (a.ldd > 0x7fffffffLL) continue;
        const int64_t pitch = tile_pitch(st, a);
        if (pitch < 0) continue;
        groups[std::make_tuple(find((int32_t)i), a.rows, a.cols, a.dst_buf, sb, pitch)].push_back((int32_t)i);
    }
    // per group (in parallel): its source list and the BF16 slices of its
    // coefficient matrix; then (in group order) the tables are appended
    struct Prep {
        bool keep = false;
        std::vector<int64_t> srcs;
        std::vector<uint8_t> wimg;   // constant image, offsets relative to its own start
        int64_t S = 0, KC = 0;
        int32_t G = 0, Gb = 0;
    };
    std::vector<const std::pair<const std::tuple<int32_t, int64_t, int64_t, int32_t, int32_t, int64_t>,
                                std::vector<int32_t>>*> glist;
    for (auto& kv : groups) glist.push_back(&kv);
    std::vector<Prep> prep(glist.size());
    auto prepare = [&](size_t gi) {
        const std::vector<int32_t>& O = glist[gi]->second;
        const int64_t cols = std::get<2>(glist[gi]->first), pitch = std::get<5>(glist[gi]->first);
        const int64_t E = pitch * cols;
        if (E > 0x7fffffffLL || O.size() < 8) return;
        Prep& pr = prep[gi];
        std::unordered_map<int64_t, int32_t> sid;
        int64_t nterms = 0;
        for (int32_t o : O)
            for (int64_t k = st.aout[o].t_begin; k < st.aout[o].t_end; ++k, ++nterms)
                if (sid.emplace(st.aterm[k].src_off, (int32_t)pr.srcs.size()).second) pr.srcs.push_back(st.aterm[k].src_off);
        const int64_t S = (int64_t)pr.srcs.size();
        // dense block products pay when a fair share of the (outputs x sources) block is populated
        if ((double)nterms < 0.05 * (double)O.size() * (double)S) return;
        pr.keep = true;
        pr.S = S;
        pr.KC = (S + 31) / 32;
        pr.G = (int32_t)((E + 7) / 8);
        pr.Gb = (int32_t)((O.size() + 7) / 8);
        // coefficient matrix W (rows = outputs, K = sources), split into BF16 slices
        std::vector<double> Wd((size_t)O.size() * S, 0.0);
        for (size_t j = 0; j < O.size(); ++j)
            for (int64_t k = st.aout[O[j]].t_begin; k < st.aout[O[j]].t_end; ++k)
                Wd[j * S + sid[st.aterm[k].src_off]] += st.aterm[k].alpha;
        pr.wimg.assign((size_t)(pr.KC * 3 * (int64_t)pr.Gb * 512), 0);
        for (size_t j = 0; j < O.size(); ++j)
            for (int64_t k = 0; k < S; ++k) {
                const float x = (float)Wd[j * S + k];
                if (x == 0.0f) continue;
                const uint16_t h0 = bf16_rne(x);
                const float r1 = x - bf16_to_float(h0);
                const uint16_t h1 = bf16_rne(r1);
                const float r2 = r1 - bf16_to_float(h1);
                const uint16_t h2 = bf16_rne(r2);
                const uint16_t h[3] = {h0, h1, h2};
                const int64_t c = k / 32, q = (k % 32) / 8;
                for (int sl = 0; sl < 3; ++sl) {
                    const int64_t byte = ((c * 3 + sl) * pr.Gb + (int64_t)(j / 8)) * 512 + q * 128 +
                                         (int64_t)(j % 8) * 16 + (k % 8) * 2;
                    std::memcpy(&pr.wimg[(size_t)byte], &h[sl], 2);
                }
            }
    };
    {
        std::atomic<size_t> next{0};
        auto worker = [&]() {
            for (;;) {
                const size_t gi = next.fetch_add(1);
                if (gi >= glist.size()) return;
                prepare(gi);
            }
        };
        const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (unsigned k = 1; k < nt; ++k) pool.emplace_back(worker);
        worker();
        for (auto& th : pool) th.join();
    }
    // the groups' constant images go to their final offsets, copied in parallel
    std::vector<int64_t> cim_off(glist.size(), 0);
    {
        int64_t c = (int64_t)t.cimg.size();
        for (size_t gi = 0; gi < glist.size(); ++gi)
            if (prep[gi].keep) { cim_off[gi] = c; c += (int64_t)prep[gi].wimg.size(); }
        t.cimg.resize((size_t)c);
        std::atomic<size_t> next{0};
        auto copier = [&]() {
            for (;;) {
                const size_t gi = next.fetch_add(1);
                if (gi >= glist.size()) return;
                if (!prep[gi].keep) continue;
                std::memcpy(t.cimg.data() + cim_off[gi], prep[gi].wimg.data(), prep[gi].wimg.size());
                std::vector<uint8_t>().swap(prep[gi].wimg);
            }
        };
        const unsigned nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (unsigned k = 1; k < nt; ++k) pool.emplace_back(copier);
        copier();
        for (auto& th : pool) th.join();
    }
    for (size_t gi = 0; gi < glist.size(); ++gi) {
        if (!prep[gi].keep) continue;
        const std::vector<int32_t>& O = glist[gi]->second;
        const int64_t rows = std::get<1>(glist[gi]->first), cols = std::get<2>(glist[gi]->first);
        const int32_t dst_buf = std::get<3>(glist[gi]->first), src_buf = std::get<4>(glist[gi]->first);
        const int64_t pitch = std::get<5>(glist[gi]->first);
        const int64_t E = pitch * cols;
        Prep& pr = prep[gi];
        const int64_t KC = pr.KC;
        const int32_t G = pr.G, Gb = pr.Gb;
        // A: gathered source tiles, rows e, K = source index
        ImgPanel pa;
        pa.src_off = (int64_t)t.gather.size();
        pa.img_off = t.bytes;
        pa.src_buf = src_buf;
        pa.ld = 0;
        pa.R = (int32_t)E;
        pa.K = (int32_t)pr.S;
        pa.kcontig = 2;
        pa.G = G;
        t.gather.insert(t.gather.end(), pr.srcs.begin(), pr.srcs.end());
        const int32_t pid = (int32_t)t.panels.size();
        t.bytes += KC * 3 * (int64_t)G * 512;
        for (int64_t c = 0; c < KC; ++c) { t.build.push_back(pid); t.build.push_back((int32_t)c); }
        t.panels.push_back(pa);
        // B: the group's constant image (copied above)
        const int64_t b_off = cim_off[gi];
        // output: column j is output tile O[j]
        ImgOut io;
        io.c_off = 0;
        io.si = 0;
        io.sj = 0;
        io.ctab = (int64_t)t.coltab.size() / 2;
        io.c_buf = dst_buf;
        io.mrows = (int32_t)E;
        io.ncols = (int32_t)O.size();
        io.mode = 1;
        io.rows = (int32_t)pitch;
        io.pad = pitch != rows ? (int32_t)rows : 0;   // rows stored of each pitch (0: all)
        for (int32_t o : O) {
            t.coltab.push_back(st.aout[o].dst_off);
            t.coltab.push_back(st.aout[o].ldd);
        }
        const int32_t oid = (int32_t)t.outs.size();
        t.outs.push_back(io);
        // segments: 4 K-chunks (128 sources) per drain of the accumulator
        const int32_t s_begin = (int32_t)t.segs.size();
        for (int64_t c0 = 0; c0 < KC; c0 += 4) {
            ImgSeg sg;
            sg.a_img = pa.img_off + c0 * 3 * (int64_t)G * 512;
            sg.b_img = b_off + c0 * 3 * (int64_t)Gb * 512;
            sg.a_G = G;
            sg.b_G = Gb;
            sg.kc = (int32_t)std::min<int64_t>(4, KC - c0);
            sg.alpha = 1.0f;
            sg.flags = IMG_B_CONST;
            sg.a_panel = pid;
            sg.a_c0 = (int32_t)c0;
            sg.pad = 0;
            t.segs.push_back(sg);
        }
        const int32_t s_end = (int32_t)t.segs.size();
        const int32_t nnt = (int32_t)((O.size() + 127) / 128);
        const int32_t per = (int32_t)(((O.size() + nnt - 1) / nnt + 15) / 16 * 16);
        for (int32_t m0 = 0; m0 < (int32_t)E; m0 += 128)
            for (int32_t n0 = 0; n0 < (int32_t)O.size(); n0 += per) {
                ImgUnit u;
                u.out = oid;
                u.m0 = m0;
                u.n0 = n0;
                u.nt = std::min(per, ((int32_t)O.size() - n0 + 15) / 16 * 16);
                u.s_begin = s_begin;
                u.s_end = s_end;
                t.units.push_back(u);
            }
        for (int32_t o : O) heavy[o] = 1;
    }
    if (t.build.size() / 2 > 0x7fffffffULL || t.units.size() > 0x7fffffffULL)
        throw std::runtime_error("dense groups: tables too large");
}

}  // namespace qcm

// ------------------------------------------------------------------ C entry points (host part)
using namespace qcm;

extern "C" {

const char* qcm_last_error(void) { return g_err.c_str(); }
int qcm_version(void) { return 110; }

int qcm_plan_sigma(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                   const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                   const qcm_mpo_t* mpo, int32_t hermitian, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    try {
        MpoV W(mpo);
        *plan = build_sigma(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(psi),
                            read_boundary(left), read_boundary(right), W, hermitian != 0);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_sigma: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_sigma_opts(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                        const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                        const qcm_mpo_t* mpo, int32_t hermitian, const qcm_plan_opts_t* opts, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    int64_t sk = 32, dm = 64;
    int ntm = 128, k1s = 0;
    if (opts) {
        if (opts->split_k_segs > 0) sk = opts->split_k_segs;
        if (opts->dense_min_terms > 0) dm = opts->dense_min_terms;
        if (opts->n_tile_max > 0) ntm = opts->n_tile_max;
        k1s = opts->k1_schedule;
    }
    if (sk < 2 || sk > (1 << 20) || dm < 8 || ntm < 16 || ntm > 128 || ntm % 16 || (k1s != 0 && k1s != 1)) {
        set_error("qcm_plan_sigma_opts: split_k_segs must be in [2, 2^20], dense_min_terms >= 8, n_tile_max a "
                  "multiple of 16 in [16, 128], k1_schedule 0 or 1");
        *plan = nullptr;
        return QCM_E_INVALID;
    }
    try {
        MpoV W(mpo);
        *plan = build_sigma(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(psi),
                            read_boundary(left), read_boundary(right), W, hermitian != 0, sk, dm, ntm, k1s == 1);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_sigma_opts: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_boundary_left(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                           const qcm_blocks_t* mps, const qcm_boundary_t* left, const qcm_mpo_t* mpo,
                           int32_t hermitian, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    try {
        MpoV W(mpo);
        *plan = build_bleft(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(mps),
                            read_boundary(left), W, hermitian != 0);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_boundary_left: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_diagonal(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                      const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                      const qcm_mpo_t* mpo, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    try {
        MpoV W(mpo);
        *plan = build_diag(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(psi),
                           read_boundary(left), read_boundary(right), W);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_diagonal: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_zerosite(const qcm_blocks_t* bond, const qcm_boundary_t* left, const qcm_boundary_t* right,
                      const qcm_mpo_t* mpo_left, const qcm_mpo_t* mpo_right, int32_t hermitian, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    try {
        MpoV Wl(mpo_left), Wr(mpo_right);
        *plan = build_zerosite(read_blocks(bond), read_boundary(left), read_boundary(right), Wl, Wr, hermitian != 0);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_zerosite: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_energy_gradient(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                             const qcm_blocks_t* psi, const qcm_boundary_t* left, const qcm_boundary_t* right,
                             const qcm_mpo_t* mpo, int32_t hermitian, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    try {
        MpoV W(mpo);
        *plan = build_grad(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(psi),
                           read_boundary(left), read_boundary(right), W, hermitian != 0);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_energy_gradient: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

// ------------------------------------------------------------------ batching
// One plan for many independent sigma problems: every stage's task tables are the
// concatenation of the problems' tables with their offsets moved to each problem's
// slice of shared buffers -- the caller's KET/LEFT/RIGHT/OUT slices (given), the
// scratch slots and the per-stage image bytes (back to back, in problem order),
// the plans' constant images (appended).  Each stage then runs every problem's
// work in one launch.
static qcm_plan* merge_sigma_plans(qcm_plan* const* plans, int32_t n, const int64_t* caller_off) {
    if (n < 1) throw std::runtime_error("no plans to merge");
    size_t nst = 0;
    for (int32_t k = 0; k < n; ++k) {
        if (!plans[k]) throw std::runtime_error("null plan");
        if (plans[k]->kind != PK_SIGMA) throw std::runtime_error("only sigma plans can be merged");
        nst = std::max(nst, plans[k]->stages.size());
    }
    auto* P = new qcm_plan();
    P->kind = PK_SIGMA;
    // element offsets of problem k in every slot
    std::vector<std::array<int64_t, QCM_NBUF>> base(n);
    int64_t sc[3] = {0, 0, 0};
    for (int32_t k = 0; k < n; ++k) {
        base[k].fill(0);
        for (int q = 0; q < 4; ++q) base[k][q] = caller_off[4 * k + q];
        for (int q = 0; q < 3; ++q) {
            base[k][QCM_BUF_S0 + q] = sc[q];
            // problems' scratch slices start 32-byte aligned (aligned vector loads of T)
            sc[q] += (plans[k]->scratch[q] + 3) / 4 * 4;
        }
        P->out_elems = std::max(P->out_elems, base[k][QCM_BUF_OUT] + plans[k]->out_elems);
        P->gemm_flops += plans[k]->gemm_flops;
        P->axpy_flops += plans[k]->axpy_flops;
        P->axpy_bytes += plans[k]->axpy_bytes;
    }
    for (int q = 0; q < 3; ++q) P->scratch[q] = sc[q];
    for (size_t si = 0; si < nst; ++si) {
        int kind = -1;
        for (int32_t k = 0; k < n; ++k)
            if (si < plans[k]->stages.size()) {
                const int kk = plans[k]->stages[si].kind;
                if (kind >= 0 && kk != kind) throw std::runtime_error("plans to merge differ in their stages");
                kind = kk;
            }
        Stage m;
        m.kind = kind;
        if (kind == ST_ZERO) {
            int64_t any = 0;
            for (int32_t k = 0; k < n; ++k)
                if (si < plans[k]->stages.size()) {
                    const Stage& st = plans[k]->stages[si];
                    if (m.zlen == 0) m.zbuf = st.zbuf;
                    if (st.zbuf != m.zbuf || st.zoff != 0 || st.zbuf < QCM_BUF_S0 || st.zbuf > QCM_BUF_S2)
                        throw std::runtime_error("merge: unsupported clear stage");
                    any = std::max(any, st.zlen);
                }
            // clear the whole merged slot when any problem clears its slot
            m.zlen = any > 0 ? sc[m.zbuf - QCM_BUF_S0] : 0;
        } else if (kind == ST_AXPY || kind == ST_GEMM) {
            int64_t img_off = 0;
            for (int32_t k = 0; k < n; ++k) {
                if (si >= plans[k]->stages.size()) continue;
                const Stage& st = plans[k]->stages[si];
                const auto& b = base[k];
                if (st.img.ares) throw std::runtime_error("merge: A-resident image tables are not supported");
                const int64_t o0 = kind == ST_AXPY ? (int64_t)m.aout.size() : (int64_t)m.gout.size();
                if (kind == ST_AXPY) {
                    const int64_t t0 = (int64_t)m.aterm.size();
                    for (AxpyOut o : st.aout) {
                        o.dst_off += b[o.dst_buf];
                        o.t_begin += t0;
                        o.t_end += t0;
                        m.aout.push_back(o);
                    }
                    for (AxpyTerm t : st.aterm) {
                        t.src_off += b[t.src_buf];
                        m.aterm.push_back(t);
                    }
                    if (st.comp_root.size() == st.aout.size())
                        for (int32_t r : st.comp_root) m.comp_root.push_back(r + (int32_t)o0);
                    if (st.heavy.size() == st.aout.size()) m.heavy.insert(m.heavy.end(), st.heavy.begin(), st.heavy.end());
                    else m.heavy.insert(m.heavy.end(), st.aout.size(), 0);
                } else {
                    const int64_t g0 = (int64_t)m.gseg.size();
                    for (GemmOut o : st.gout) {
                        o.c_off += b[o.c_buf];
                        o.s_begin += g0;
                        o.s_end += g0;
                        m.gout.push_back(o);
                    }
                    for (GemmSeg g : st.gseg) {
                        g.a_off += b[g.a_buf];
                        g.b_off += b[g.b_buf];
                        m.gseg.push_back(g);
                    }
                }
                // image tables
                const ImgTables& it = st.img;
                ImgTables& mt = m.img;
                const int32_t p0 = (int32_t)mt.panels.size(), u0 = (int32_t)mt.outs.size();
                const int32_t s0 = (int32_t)mt.segs.size();
                const int64_t ci0 = (int64_t)mt.cimg.size();
                for (ImgPanel pa : it.panels) {
                    if (pa.kcontig == 2) {
                        for (int32_t q = 0; q < pa.K; ++q) mt.gather.push_back(it.gather[pa.src_off + q] + b[pa.src_buf]);
                        pa.src_off = (int64_t)mt.gather.size() - pa.K;
                    } else {
                        pa.src_off += b[pa.src_buf];
                    }
                    pa.img_off += img_off;
                    mt.panels.push_back(pa);
                }
                for (size_t q = 0; q < it.build.size(); q += 2) {
                    mt.build.push_back(it.build[q] + p0);
                    mt.build.push_back(it.build[q + 1]);
                }
                for (ImgOut o : it.outs) {
                    if (o.mode == 1) {
                        for (int32_t j = 0; j < o.ncols; ++j) {
                            mt.coltab.push_back(it.coltab[2 * (o.ctab + j)] + b[o.c_buf]);
                            mt.coltab.push_back(it.coltab[2 * (o.ctab + j) + 1]);
                        }
                        o.ctab = (int64_t)mt.coltab.size() / 2 - o.ncols;
                    } else {
                        o.c_off += b[o.c_buf];
                    }
                    mt.outs.push_back(o);
                }
                for (ImgSeg sg : it.segs) {
                    sg.a_img += img_off;
                    sg.b_img += (sg.flags & IMG_B_CONST) ? ci0 : img_off;
                    sg.a_panel += p0;
                    mt.segs.push_back(sg);
                }
                for (ImgUnit u : it.units) {
                    u.out += u0;
                    u.s_begin += s0;
                    u.s_end += s0;
                    mt.units.push_back(u);
                }
                mt.cimg.insert(mt.cimg.end(), it.cimg.begin(), it.cimg.end());
                img_off += it.bytes;
            }
            m.img.bytes = img_off;
            P->image_bytes = std::max(P->image_bytes, img_off);
            if (kind == ST_AXPY && m.comp_root.size() != m.aout.size()) m.comp_root.clear();
        } else {
            throw std::runtime_error("merge: unsupported stage kind");
        }
        P->stages.push_back(std::move(m));
    }
    return P;
}

int qcm_plan_merge(qcm_plan* const* plans, int32_t n, const int64_t* caller_off, qcm_plan** out) {
    if (!out || !plans || !caller_off) { set_error("null argument"); return QCM_E_INVALID; }
    try {
        *out = merge_sigma_plans(plans, n, caller_off);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_merge: ") + e.what());
        *out = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_boundary_tensor_mpo(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                                 const qcm_blocks_t* mps, const qcm_boundary_t* boundary, const qcm_mpo_t* mpo,
                                 int32_t side, int32_t hermitian, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    if (side != 0 && side != 1) { set_error("qcm_plan_boundary_tensor_mpo: side must be 0 (left) or 1 (right)"); return QCM_E_INVALID; }
    try {
        MpoV W(mpo);
        if (side == 0)
            *plan = build_bleft(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(mps),
                                read_boundary(boundary), W, hermitian != 0, true);
        else
            *plan = build_bright(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(mps),
                                 read_boundary(boundary), W, hermitian != 0, true);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_boundary_tensor_mpo: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_boundary_right(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                            const qcm_blocks_t* mps, const qcm_boundary_t* right, const qcm_mpo_t* mpo,
                            int32_t hermitian, qcm_plan** plan) {
    if (!plan) { set_error("null plan pointer"); return QCM_E_INVALID; }
    try {
        MpoV W(mpo);
        *plan = build_bright(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(mps),
                             read_boundary(right), W, hermitian != 0);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_plan_boundary_right: ") + e.what());
        *plan = nullptr;
        return QCM_E_INVALID;
    }
}

int qcm_plan_sizes(const qcm_plan* p, int64_t* out_elems, int64_t* scratch3) {
    if (!p) { set_error("null plan"); return QCM_E_INVALID; }
    if (out_elems) *out_elems = p->out_elems;
    if (scratch3) for (int i = 0; i < 3; ++i) scratch3[i] = p->scratch[i];
    return QCM_OK;
}

int qcm_plan_stage_images(const qcm_plan* p, int32_t stage, int64_t* counts, int64_t* pd, int64_t* od,
                          int64_t* sd, double* sa, int64_t* td) {
    if (!p || !counts) { set_error("null argument"); return QCM_E_INVALID; }
    if (stage < 0 || stage >= (int32_t)p->stages.size()) { set_error("stage out of range"); return QCM_E_RANGE; }
    const ImgTables& t = p->stages[stage].img;
    counts[0] = (int64_t)t.panels.size();
    counts[1] = (int64_t)t.outs.size();
    counts[2] = (int64_t)t.segs.size();
    counts[3] = (int64_t)t.units.size();
    if (pd)
        for (size_t i = 0; i < t.panels.size(); ++i) {
            const ImgPanel& x = t.panels[i];
            const int64_t v[8] = {x.src_off, x.img_off, x.src_buf, x.ld, x.R, x.K, x.kcontig, x.G};
            for (int j = 0; j < 8; ++j) pd[8 * i + j] = v[j];
        }
    if (od)
        for (size_t i = 0; i < t.outs.size(); ++i) {
            const ImgOut& x = t.outs[i];
            const int64_t v[10] = {x.c_off, x.si, x.sj, x.c_buf, x.mrows, x.ncols, x.mode, x.rows, x.ctab, x.pad};
            for (int j = 0; j < 10; ++j) od[10 * i + j] = v[j];
        }
    if (sd)
        for (size_t i = 0; i < t.segs.size(); ++i) {
            const ImgSeg& x = t.segs[i];
            const int64_t v[8] = {x.a_img, x.b_img, x.a_G, x.b_G, x.kc, x.flags, x.a_panel, x.a_c0};
            for (int j = 0; j < 8; ++j) sd[8 * i + j] = v[j];
            if (sa) sa[i] = x.alpha;
        }
    if (td)
        for (size_t i = 0; i < t.units.size(); ++i) {
            const ImgUnit& x = t.units[i];
            const int64_t v[6] = {x.out, x.m0, x.n0, x.nt, x.s_begin, x.s_end};
            for (int j = 0; j < 6; ++j) td[6 * i + j] = v[j];
        }
    return QCM_OK;
}

int qcm_plan_stage_image_aux(const qcm_plan* p, int32_t stage, int64_t* counts, int64_t* gather, int64_t* coltab,
                             uint8_t* cimg) {
    if (!p || !counts) { set_error("null argument"); return QCM_E_INVALID; }
    if (stage < 0 || stage >= (int32_t)p->stages.size()) { set_error("stage out of range"); return QCM_E_RANGE; }
    const ImgTables& t = p->stages[stage].img;
    counts[0] = (int64_t)t.gather.size();
    counts[1] = (int64_t)t.coltab.size();
    counts[2] = (int64_t)t.cimg.size();
    if (gather && !t.gather.empty()) std::memcpy(gather, t.gather.data(), t.gather.size() * 8);
    if (coltab && !t.coltab.empty()) std::memcpy(coltab, t.coltab.data(), t.coltab.size() * 8);
    if (cimg && !t.cimg.empty()) std::memcpy(cimg, t.cimg.data(), t.cimg.size());
    return QCM_OK;
}

int qcm_plan_last_kernels(const qcm_plan* p, int32_t* n) {
    if (!p || !n) { set_error("null argument"); return QCM_E_INVALID; }
    *n = p->last_kernels;
    return QCM_OK;
}

int qcm_plan_image_bytes(const qcm_plan* p, int64_t* bytes) {
    if (!p || !bytes) { set_error("null argument"); return QCM_E_INVALID; }
    *bytes = p->image_bytes;
    return QCM_OK;
}

int qcm_plan_work(const qcm_plan* p, double* gf, double* af, double* ab, int32_t* launches) {
    if (!p) { set_error("null plan"); return QCM_E_INVALID; }
    if (gf) *gf = p->gemm_flops;
    if (af) *af = p->axpy_flops;
    if (ab) *ab = p->axpy_bytes;
    if (launches) {
        int n = 0;
        for (auto& s : p->stages) {
            if (s.kind == ST_ZERO) { if (s.zlen > 0) ++n; }
            else if ((s.kind == ST_AXPY && !s.aout.empty()) || (s.kind == ST_GEMM && !s.gout.empty())) ++n;
        }
        *launches = n;
    }
    return QCM_OK;
}

int qcm_plan_out_layout(const qcm_plan* p, int32_t* aux, int32_t* nblocks, int32_t* blk_ptr, int32_t* q,
                        int64_t* rows, int64_t* cols, int64_t* off) {
    if (!p) { set_error("null plan"); return QCM_E_INVALID; }
    if (p->kind == PK_SIGMA) { set_error("sigma plans have no boundary output layout"); return QCM_E_STATE; }
    if (aux) *aux = (int32_t)p->out_blk_ptr.size() - 1;
    if (nblocks) *nblocks = (int32_t)p->out_blocks.size();
    if (blk_ptr) for (size_t i = 0; i < p->out_blk_ptr.size(); ++i) blk_ptr[i] = p->out_blk_ptr[i];
    for (size_t k = 0; k < p->out_blocks.size(); ++k) {
        const Blk& b = p->out_blocks[k];
        if (q) { q[4 * k] = b.lc.n; q[4 * k + 1] = b.lc.s; q[4 * k + 2] = b.rc.n; q[4 * k + 3] = b.rc.s; }
        if (rows) rows[k] = b.rows;
        if (cols) cols[k] = b.cols;
        if (off) off[k] = b.off;
    }
    return QCM_OK;
}

int qcm_plan_num_stages(const qcm_plan* p, int32_t* n) {
    if (!p || !n) { set_error("null argument"); return QCM_E_INVALID; }
    *n = (int32_t)p->stages.size();
    return QCM_OK;
}

int qcm_plan_stage_info(const qcm_plan* p, int32_t s, int32_t* kind, int64_t* n_out, int64_t* n_terms) {
    if (!p || s < 0 || s >= (int32_t)p->stages.size()) { set_error("bad stage"); return QCM_E_INVALID; }
    const Stage& st = p->stages[s];
    if (kind) *kind = st.kind;
    if (st.kind == ST_AXPY) {
        if (n_out) *n_out = (int64_t)st.aout.size();
        if (n_terms) *n_terms = (int64_t)st.aterm.size();
    } else if (st.kind == ST_GEMM) {
        if (n_out) *n_out = (int64_t)st.gout.size();
        if (n_terms) *n_terms = (int64_t)st.gseg.size();
    } else if (st.kind == ST_DOT) {
        if (n_out) *n_out = (int64_t)st.aout.size();
        if (n_terms) *n_terms = (int64_t)st.aterm.size();
    } else {
        if (n_out) *n_out = st.zbuf;
        if (n_terms) *n_terms = st.zlen;
    }
    return QCM_OK;
}

int qcm_plan_stage_dot(const qcm_plan* p, int32_t s, int64_t* od, int64_t* td, double* w, int32_t* tt,
                       int32_t* meta) {
    if (!p || s < 0 || s >= (int32_t)p->stages.size() || p->stages[s].kind != ST_DOT) {
        set_error("not a dot stage");
        return QCM_E_INVALID;
    }
    const Stage& st = p->stages[s];
    if (meta) { meta[0] = st.dot_buf; meta[1] = st.n_tt; }
    for (size_t i = 0; i < st.aout.size(); ++i) {
        const AxpyOut& o = st.aout[i];
        int64_t* d = od + 7 * i;
        d[0] = o.dst_buf; d[1] = o.dst_off; d[2] = o.ldd; d[3] = o.rows; d[4] = o.cols; d[5] = o.t_begin; d[6] = o.t_end;
    }
    for (size_t i = 0; i < st.aterm.size(); ++i) {
        td[3 * i] = st.aterm[i].src_buf;
        td[3 * i + 1] = st.aterm[i].src_off;
        td[3 * i + 2] = st.aterm[i].lds;
        w[i] = st.dot_w[i];
        tt[i] = st.dot_tt[i];
    }
    return QCM_OK;
}

int qcm_plan_stage_axpy(const qcm_plan* p, int32_t s, int64_t* od, int64_t* td, double* ta) {
    if (!p || s < 0 || s >= (int32_t)p->stages.size() || p->stages[s].kind != ST_AXPY) {
        set_error("not an axpy stage");
        return QCM_E_INVALID;
    }
    const Stage& st = p->stages[s];
    for (size_t i = 0; i < st.aout.size(); ++i) {
        const AxpyOut& o = st.aout[i];
        int64_t* d = od + 7 * i;
        d[0] = o.dst_buf; d[1] = o.dst_off; d[2] = o.ldd; d[3] = o.rows; d[4] = o.cols; d[5] = o.t_begin; d[6] = o.t_end;
    }
    for (size_t i = 0; i < st.aterm.size(); ++i) {
        td[3 * i] = st.aterm[i].src_buf;
        td[3 * i + 1] = st.aterm[i].src_off;
        td[3 * i + 2] = st.aterm[i].lds;
        ta[i] = st.aterm[i].alpha;
    }
    return QCM_OK;
}

int qcm_plan_stage_gemm(const qcm_plan* p, int32_t s, int64_t* od, int64_t* sd, double* sa) {
    if (!p || s < 0 || s >= (int32_t)p->stages.size() || p->stages[s].kind != ST_GEMM) {
        set_error("not a gemm stage");
        return QCM_E_INVALID;
    }
    const Stage& st = p->stages[s];
    for (size_t i = 0; i < st.gout.size(); ++i) {
        const GemmOut& o = st.gout[i];
        int64_t* d = od + 7 * i;
        d[0] = o.c_buf; d[1] = o.c_off; d[2] = o.ldc; d[3] = o.M; d[4] = o.N; d[5] = o.s_begin; d[6] = o.s_end;
    }
    for (size_t i = 0; i < st.gseg.size(); ++i) {
        const GemmSeg& g = st.gseg[i];
        int64_t* d = sd + 9 * i;
        d[0] = g.a_buf; d[1] = g.ta; d[2] = g.a_off; d[3] = g.lda; d[4] = g.b_buf; d[5] = g.tb; d[6] = g.b_off;
        d[7] = g.ldb; d[8] = g.K;
        sa[i] = g.alpha;
    }
    return QCM_OK;
}

void qcm_plan_destroy(qcm_plan* p) {
    if (!p) return;
    release_plan_device(p);
    delete p;
}

}  // extern "C"
