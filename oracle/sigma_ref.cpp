// C++17 / OpenMP restatement of the reference's lbtm sigma vector (oracle; test
// infrastructure and the timed CPU baseline -- never part of the library).
//
// site_hamil_lbtm (dmrg/framework/dmrg/mp_tensors/contractions/non-abelian/
// site_hamil.hpp:57-147), for bra = ket:
//   1. the ket reshaped to right-paired (reshape_left_to_right_new,
//      mp_tensors/reshapes.h);
//   2. T[b1] = op(L[b1]) . ket for every left MPO bond b1, trimmed to the ket's
//      left charges (BoundaryMPSProduct with SU2::gemm_trim_left,
//      ct/common/boundary_times_mps.hpp:163-209, ct/non-abelian/gemm.hpp:78-115);
//      a Hermitian-skipped b1 reads its partner's block untransposed, scaled by
//      conjugate_correction x the bond phase (boundary_times_mps.hpp:19-43);
//   3. for every right bond b2 (OpenMP over b2, as the reference's loop at
//      site_hamil.hpp:115-144): contr = lbtm_kernel (ct/non-abelian/
//      apply_op.hpp:23-101 with the micro-axpys of micro_kernels.hpp:19-45 and
//      the SU(2) couplings of set_coupling, bm/symmetry/gsl_coupling.h:175-204),
//      then sigma += gemm_trim(contr, R[b2]) (gemm.hpp:178-204), R[b2] taken from
//      its Hermitian partner (transposed, with phases) where b2 is skipped.
// Each thread accumulates into its own sigma; the thread partials are added in
// thread order at the end (the reference adds under a critical section).
//
// Block products call a BLAS dgemm through a function pointer (the host's
// OpenBLAS, ILP64 CBLAS interface, set single-threaded inside the OpenMP
// region), or this file's own cache-blocked loop nest when none is given.  The
// 9j symbols are Racah sums in long double.  Work counters: 2mnk per block
// product, 2 x (rows x cols) per micro-axpy, as the GPU plans count them.
//
// Inputs use the plain layout structs of the library's C ABI header (the ABI's
// data format, shared by design); nothing of the library is linked or called.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <tuple>
#include <vector>

#include "qcm_gb300.h"

namespace {

struct Ch {
    int n = 0, s = 0;
    bool operator<(const Ch& o) const { return n != o.n ? n < o.n : s < o.s; }
    bool operator==(const Ch& o) const { return n == o.n && s == o.s; }
    bool operator!=(const Ch& o) const { return !(*this == o); }
    bool operator>(const Ch& o) const { return o < *this; }
};
Ch add(Ch a, Ch b) { return {a.n + b.n, a.s + b.s}; }
Ch minus(Ch a) { return {-a.n, -a.s}; }
bool tri(int a, int b, int c) { return (a + b + c) % 2 == 0 && std::abs(a - b) <= c && c <= a + b; }

struct Idx {
    std::vector<std::pair<Ch, int64_t>> e;   // descending charges
    int pos(Ch c) const {
        for (size_t k = 0; k < e.size(); ++k)
            if (e[k].first == c) return (int)k;
        return -1;
    }
    void add_or_insert(Ch c, int64_t s) {
        int p = pos(c);
        if (p >= 0) { e[p].second += s; return; }
        size_t k = 0;
        while (k < e.size() && !(e[k].first < c)) ++k;
        e.insert(e.begin() + k, {c, s});
    }
};

// offsets of (a, b) pairs inside their fused sector, a outer, b inner
struct PBasis {
    std::map<std::pair<std::pair<int, int>, std::pair<int, int>>, int64_t> off;
    std::map<std::pair<int, int>, int64_t> size;
    PBasis(const Idx& a, const Idx& b, bool neg_a) {
        for (auto& x : a.e)
            for (auto& y : b.e) {
                Ch f = add(neg_a ? minus(x.first) : x.first, y.first);
                auto key = std::make_pair(f.n, f.s);
                int64_t& cur = size[key];
                off[{{x.first.n, x.first.s}, {y.first.n, y.first.s}}] = cur;
                cur += x.second * y.second;
            }
    }
    int64_t at(Ch a, Ch b) const { return off.at({{a.n, a.s}, {b.n, b.s}}); }
};

// a dense block, column-major; data either owned or a view
struct Blk {
    Ch l, r;
    int64_t rows = 0, cols = 0;
    const double* view = nullptr;
    std::vector<double> own;
    const double* ptr() const { return view ? view : own.data(); }
    double* mut() { return own.data(); }
};
struct BMat {
    std::vector<Blk> b;   // descending (l, r)
    int find(Ch l, Ch r) const {
        for (size_t k = 0; k < b.size(); ++k)
            if (b[k].l == l && b[k].r == r) return (int)k;
        return -1;
    }
    Blk& get_or_zero(Ch l, Ch r, int64_t rows, int64_t cols) {
        int k = find(l, r);
        if (k >= 0) return b[k];
        Blk x;
        x.l = l;
        x.r = r;
        x.rows = rows;
        x.cols = cols;
        x.own.assign((size_t)rows * cols, 0.0);
        size_t p = 0;
        while (p < b.size() && (b[p].l > l || (b[p].l == l && b[p].r > r))) ++p;
        b.insert(b.begin() + p, std::move(x));
        return b[p];
    }
};

using dgemm_fn = void (*)(int, int, int, int64_t, int64_t, int64_t, double, const double*, int64_t, const double*,
                          int64_t, double, double*, int64_t);
dgemm_fn g_gemm = nullptr;

// C (m x n) += alpha op(A) op(B), column-major; ta/tb: 0 plain, 1 transposed
void gemm(int ta, int tb, int64_t m, int64_t n, int64_t k, double alpha, const double* A, int64_t lda,
          const double* B, int64_t ldb, double* C, int64_t ldc) {
    if (m == 0 || n == 0 || k == 0) return;
    if (g_gemm) {
        g_gemm(102, ta ? 112 : 111, tb ? 112 : 111, m, n, k, alpha, A, lda, B, ldb, 1.0, C, ldc);
        return;
    }
    auto a = [&](int64_t i, int64_t p) { return ta ? A[p + i * lda] : A[i + p * lda]; };
    auto bb = [&](int64_t p, int64_t j) { return tb ? B[j + p * ldb] : B[p + j * ldb]; };
    const int64_t bs = 64;
    for (int64_t j0 = 0; j0 < n; j0 += bs)
        for (int64_t p0 = 0; p0 < k; p0 += bs)
            for (int64_t j = j0; j < std::min(n, j0 + bs); ++j)
                for (int64_t p = p0; p < std::min(k, p0 + bs); ++p) {
                    const double s = alpha * bb(p, j);
                    double* c = C + j * ldc;
                    for (int64_t i = 0; i < m; ++i) c[i] += s * a(i, p);
                }
}

// ---- SU(2) couplings (Racah sums; mod_coupling / set_coupling)
long double lf(int n) {
    static std::vector<long double> t = [] {
        std::vector<long double> v(400);
        v[0] = 0.0L;
        for (int i = 1; i < 400; ++i) v[i] = v[i - 1] + std::log((long double)i);
        return v;
    }();
    return t.at(n);
}
long double tri_ln(int a, int b, int c) {
    return 0.5L * (lf((a + b - c) / 2) + lf((a - b + c) / 2) + lf((-a + b + c) / 2) - lf((a + b + c) / 2 + 1));
}
long double six_j(int a, int b, int c, int d, int e, int f) {
    if (!tri(a, b, c) || !tri(a, e, f) || !tri(d, b, f) || !tri(d, e, c)) return 0.0L;
    const int t1 = (a + b + c) / 2, t2 = (a + e + f) / 2, t3 = (d + b + f) / 2, t4 = (d + e + c) / 2;
    const int q1 = (a + b + d + e) / 2, q2 = (b + c + e + f) / 2, q3 = (a + c + d + f) / 2;
    const long double pre = tri_ln(a, b, c) + tri_ln(a, e, f) + tri_ln(d, b, f) + tri_ln(d, e, c);
    long double s = 0.0L;
    for (int t = std::max({t1, t2, t3, t4}); t <= std::min({q1, q2, q3}); ++t) {
        long double ln = lf(t + 1) - lf(t - t1) - lf(t - t2) - lf(t - t3) - lf(t - t4) - lf(q1 - t) - lf(q2 - t) -
                         lf(q3 - t) + pre;
        s += (t % 2 ? -1.0L : 1.0L) * std::exp(ln);
    }
    return s;
}
long double nine_j(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    // {a b c; d e f; g h i} = sum_x (-1)^2x (2x+1) {a b c; f i x} {d e f; b x h} {g h i; x a d}
    long double s = 0.0L;
    for (int x = std::max({std::abs(a - i), std::abs(b - f), std::abs(d - h)}); x <= std::min({a + i, b + f, d + h});
         x += 2)
        s += (x % 2 ? -1.0L : 1.0L) * (x + 1) * six_j(a, b, c, f, i, x) * six_j(d, e, f, b, x, h) *
             six_j(g, h, i, x, a, d);
    return s;
}
double mod_coupling(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    return (double)(std::sqrt((long double)(g + 1) * (h + 1) * (c + 1) * (f + 1)) * nine_j(a, b, c, d, e, f, g, h, i));
}
std::mutex g_cpl_mu;
std::map<std::vector<int>, std::vector<double>> g_cpl;
// the four couplings of one MPO entry (times init), cached on the spin arguments
void couplings(int a, int b, int c, int d, int e, int f, int g, int h, int i, double init, double out[4]) {
    std::vector<int> key = {a, b, c, d, e, f, g, h, i};
    std::vector<double> v;
    {
        std::lock_guard<std::mutex> lk(g_cpl_mu);
        auto it = g_cpl.find(key);
        if (it != g_cpl.end()) v = it->second;
    }
    if (v.empty()) {
        v.assign(4, 0.0);
        const double pre = std::sqrt((i + 1.0) * (a + 1.0) / ((g + 1.0) * (c + 1.0)));
        if (tri(a, b, c)) {
            v[0] = pre * mod_coupling(a, b, c, d, e, f, g, h, i);
            v[2] = pre * mod_coupling(a, b, c, d, e, f, g, 2, i);
        }
        if (tri(a, 2, c)) {
            v[1] = pre * mod_coupling(a, 2, c, d, e, f, g, h, i);
            v[3] = pre * mod_coupling(a, 2, c, d, e, f, g, 2, i);
        }
        std::lock_guard<std::mutex> lk(g_cpl_mu);
        g_cpl[key] = v;
    }
    for (int k = 0; k < 4; ++k) out[k] = v[k] * init;
}
double conj_corr(int lcs, int rcs, int S) {
    const double m = std::min(lcs, rcs);
    const int diff = rcs - lcs;
    if (S == 0) return 1.0;
    if (S == 1) return diff > 0 ? -std::sqrt((m + 1.0) / (m + 2.0)) : (diff < 0 ? std::sqrt((m + 2.0) / (m + 1.0)) : 0.0);
    if (S == 2) return diff > 0 ? -std::sqrt((m + 1.0) / (m + 3.0)) : (diff < 0 ? -std::sqrt((m + 3.0) / (m + 1.0)) : 1.0);
    throw std::runtime_error("conjugate correction for rank > 1");
}

Idx read_idx(const qcm_index_t* x) {
    Idx r;
    for (int k = 0; k < x->n; ++k) r.e.push_back({{x->q[2 * k], x->q[2 * k + 1]}, x->size[k]});
    return r;
}
BMat view_blocks(int n, const int32_t* q, const int64_t* rows, const int64_t* cols, const int64_t* off,
                 const double* data) {
    BMat m;
    for (int k = 0; k < n; ++k) {
        Blk b;
        b.l = {q[4 * k], q[4 * k + 1]};
        b.r = {q[4 * k + 2], q[4 * k + 3]};
        b.rows = rows[k];
        b.cols = cols[k];
        b.view = data + off[k];
        m.b.push_back(std::move(b));
    }
    return m;
}

struct Sparse { int r, c, rs, cs; double v; };

}  // namespace

extern "C" {

// sigma (ket layout, FP64) = H_eff ket; returns 0, or -1 with a message in err.
int oracle_sigma(const qcm_index_t* phys_c, const qcm_index_t* left_c, const qcm_index_t* right_c,
                 const qcm_blocks_t* psi_c, const double* psi, const qcm_boundary_t* Lc, const double* Ld,
                 const qcm_boundary_t* Rc, const double* Rd, const qcm_mpo_t* W, int32_t hermitian, double* sigma,
                 double* work3, void* dgemm_ptr, int32_t threads, char* err, int32_t err_len) {
    try {
        g_gemm = (dgemm_fn)dgemm_ptr;
        if (threads > 0) omp_set_num_threads(threads);
        const Idx phys = read_idx(phys_c), left_i = read_idx(left_c), right_i = read_idx(right_c);
        BMat ket = view_blocks(psi_c->n, psi_c->q, psi_c->rows, psi_c->cols, psi_c->off, psi);
        auto bnd = [](const qcm_boundary_t* c, const double* d) {
            std::vector<BMat> v(c->aux);
            for (int b = 0; b < c->aux; ++b)
                v[b] = view_blocks(c->blk_ptr[b + 1] - c->blk_ptr[b], c->q + 4 * c->blk_ptr[b], c->rows + c->blk_ptr[b],
                                   c->cols + c->blk_ptr[b], c->off + c->blk_ptr[b], d);
            return v;
        };
        std::vector<BMat> L = bnd(Lc, Ld), R = bnd(Rc, Rd);
        // out_left_i = phys x left, restricted to the right index's charges
        Idx out_left;
        for (auto& p : phys.e)
            for (auto& l : left_i.e) out_left.add_or_insert(add(p.first, l.first), p.second * l.second);
        std::sort(out_left.e.begin(), out_left.e.end(), [](auto& x, auto& y) { return x.first > y.first; });
        {
            Idx keep;
            for (auto& e : out_left.e)
                if (right_i.pos(e.first) >= 0) keep.e.push_back(e);
            out_left = keep;
        }
        const PBasis out_left_pb(phys, left_i, false), in_right_pb(phys, right_i, true);
        // 1. ket right-paired: block (l, -s + r) of rows l, columns (s, r)
        BMat rp;
        for (auto& blk : ket.b) {
            const int r = right_i.pos(blk.r);
            if (r < 0) continue;
            for (auto& ps : phys.e) {
                const int l = left_i.pos(add(blk.l, minus(ps.first)));
                if (l < 0) continue;
                const Ch ol = left_i.e[l].first, orr = add(minus(ps.first), right_i.e[r].first);
                const int64_t ld = left_i.e[l].second, rd = right_i.e[r].second;
                Blk& ob = rp.get_or_zero(ol, orr, ld, in_right_pb.size.at({orr.n, orr.s}));
                const int64_t ilo = out_left_pb.at(ps.first, ol), oro = in_right_pb.at(ps.first, right_i.e[r].first);
                for (int64_t ss = 0; ss < ps.second; ++ss)
                    for (int64_t c = 0; c < rd; ++c)
                        for (int64_t i = 0; i < ld; ++i)
                            ob.mut()[i + (oro + ss * rd + c) * ob.rows] =
                                blk.ptr()[ilo + ss * ld + i + c * blk.rows];
            }
        }
        std::vector<Ch> ref;
        for (auto& b : rp.b) ref.push_back(b.l);
        auto in_ref = [&](Ch c) { return std::find(ref.begin(), ref.end(), c) != ref.end(); };
        // MPO views
        const int D1 = W->row_dim, D2 = W->col_dim;
        std::vector<std::vector<int>> col_b1(D2), col_e(D2);
        for (int b2 = 0; b2 < D2; ++b2)
            for (int e = W->col_ptr[b2]; e < W->col_ptr[b2 + 1]; ++e) {
                col_b1[b2].push_back(W->row_of[e]);
                col_e[b2].push_back(e);
            }
        // operator sparse entries per block
        std::vector<std::vector<std::pair<std::pair<Ch, Ch>, std::vector<Sparse>>>> ops(W->n_ops);
        for (int o = 0; o < W->n_ops; ++o)
            for (int k = W->op_blk_ptr[o]; k < W->op_blk_ptr[o + 1]; ++k) {
                std::vector<Sparse> es;
                for (int en = W->blk_ent_ptr[k]; en < W->blk_ent_ptr[k + 1]; ++en)
                    es.push_back({W->ent[4 * en], W->ent[4 * en + 1], W->ent[4 * en + 2], W->ent[4 * en + 3],
                                  W->ent_coeff[en]});
                ops[o].push_back({{{W->blk_q[4 * k], W->blk_q[4 * k + 1]}, {W->blk_q[4 * k + 2], W->blk_q[4 * k + 3]}},
                                  es});
            }
        double gemm_flops = 0, axpy_flops = 0;
        // 2. T[b1] = op(L[b1]) . rp over the ket's left charges
        std::vector<BMat> T(L.size());
#pragma omp parallel for schedule(dynamic) reduction(+ : gemm_flops)
        for (int b1 = 0; b1 < (int)L.size(); ++b1) {
            const bool conj = hermitian && b1 < D1 && W->left_herm[b1] < b1;
            const BMat& src = conj ? L[W->left_herm[b1]] : L[b1];
            struct A { Ch l, r; const double* p; int64_t ld, m, k; int t; double s; };
            std::vector<A> as;
            for (auto& x : src.b) {
                if (conj)
                    as.push_back({x.l, x.r, x.ptr(), x.rows, x.rows, x.cols, 0,
                                  conj_corr(x.l.s, x.r.s, W->left_spin[b1]) * W->left_phase[b1]});
                else
                    as.push_back({x.r, x.l, x.ptr(), x.rows, x.cols, x.rows, 1, 1.0});
            }
            std::stable_sort(as.begin(), as.end(), [](const A& p, const A& q) {
                return p.l > q.l || (p.l == q.l && p.r > q.r);
            });
            for (auto& a : as) {
                if (!in_ref(a.l)) continue;
                for (auto& rb : rp.b) {
                    if (rb.l != a.r) continue;
                    Blk& c = T[b1].get_or_zero(a.l, rb.r, a.m, rb.cols);
                    gemm(a.t, 0, a.m, rb.cols, a.k, a.s, a.p, a.ld, rb.ptr(), rb.rows, c.mut(), c.rows);
                    gemm_flops += 2.0 * a.m * rb.cols * a.k;
                }
            }
        }
        // 3. per b2: contr = lbtm_kernel, sigma += gemm_trim(contr, R[b2])
        const int nth = omp_get_max_threads();
        std::vector<BMat> part(nth);
#pragma omp parallel for schedule(dynamic) reduction(+ : gemm_flops, axpy_flops)
        for (int b2 = 0; b2 < D2; ++b2) {
            BMat& acc = part[omp_get_thread_num()];
            BMat contr;
            const int ap = W->right_spin[b2];
            for (size_t ie = 0; ie < col_b1[b2].size(); ++ie) {
                const int b1 = col_b1[b2][ie], e = col_e[b2][ie];
                const BMat& Tb = T[b1];
                const int a = W->left_spin[b1];
                for (int t = W->term_ptr[e]; t < W->term_ptr[e + 1]; ++t) {
                    const int op = W->term_op[t], k = W->op_spin[op];
                    const double scale = W->term_scale[t];
                    for (auto& tb : Tb.b) {
                        const Ch lc = tb.l, rc = tb.r;
                        for (auto& wb : ops[op]) {
                            const Ch pin = wb.first.first, pout = wb.first.second;
                            const Ch out_r = add(rc, pin);
                            const int rb = right_i.pos(out_r);
                            if (rb < 0) continue;
                            const Ch out_l = add(lc, pout);
                            if (!tri(out_r.s, ap, out_l.s)) continue;
                            const int ol = out_left.pos(out_l);
                            if (ol < 0) continue;
                            const int64_t r_size = right_i.e[rb].second, l_size = tb.rows;
                            Blk& ob = contr.get_or_zero(out_l, out_r, out_left.e[ol].second, r_size);
                            const int i = lc.s, ip = out_l.s, j = rc.s, jp = out_r.s;
                            double cpl[4];
                            couplings(j, std::abs(j - jp), jp, a, k, ap, i, std::abs(i - ip), ip, scale, cpl);
                            const int64_t iro = in_right_pb.at(pin, out_r), olo = out_left_pb.at(pout, lc);
                            for (auto& s : wb.second) {
                                const int cs = (s.rs == 2 && s.cs == 2) ? 3 : (s.rs == 2 ? 1 : (s.cs == 2 ? 2 : 0));
                                const double alfa = s.v * cpl[cs];
                                for (int64_t c = 0; c < r_size; ++c) {
                                    double* dst = ob.mut() + olo + s.c * l_size + c * ob.rows;
                                    const double* src = tb.ptr() + (iro + s.r * r_size + c) * tb.rows;
                                    for (int64_t x = 0; x < l_size; ++x) dst[x] += alfa * src[x];
                                }
                                axpy_flops += 2.0 * l_size * r_size;
                            }
                        }
                    }
                }
            }
            const bool skip = hermitian && W->right_herm[b2] < b2;
            const BMat& Rb = skip ? R[W->right_herm[b2]] : R[b2];
            const double ph = skip ? W->right_phase[W->right_herm[b2]] : 1.0;
            for (auto& cb : contr.b) {
                // the R block (ar, al), or the partner's (al, ar) transposed
                const int m = skip ? Rb.find(cb.l, cb.r) : Rb.find(cb.r, cb.l);
                if (m < 0) continue;
                const Blk& rbk = Rb.b[m];
                const double s = skip ? conj_corr(cb.r.s, cb.l.s, ap) * ph : 1.0;
                const int64_t ncol = skip ? rbk.rows : rbk.cols;
                Blk& o = acc.get_or_zero(cb.l, cb.l, cb.rows, ncol);
                gemm(0, skip ? 1 : 0, cb.rows, ncol, cb.cols, s, cb.ptr(), cb.rows, rbk.ptr(), rbk.rows, o.mut(),
                     o.rows);
                gemm_flops += 2.0 * cb.rows * ncol * cb.cols;
            }
        }
        // thread partials in thread order into the ket's layout
        for (int k = 0; k < psi_c->n; ++k) std::fill(sigma + psi_c->off[k], sigma + psi_c->off[k] + psi_c->rows[k] *
                                                                                         psi_c->cols[k], 0.0);
        for (auto& p : part)
            for (auto& b : p.b) {
                int k = ket.find(b.l, b.r);
                if (k < 0) continue;
                if (b.rows != ket.b[k].rows || b.cols != ket.b[k].cols)
                    throw std::runtime_error("sigma block shape differs from the ket's");
                double* dst = sigma + psi_c->off[k];
                for (int64_t x = 0; x < b.rows * b.cols; ++x) dst[x] += b.own[x];
            }
        if (work3) {
            work3[0] = gemm_flops;
            work3[1] = axpy_flops;
            work3[2] = (double)nth;
        }
        return 0;
    } catch (const std::exception& e) {
        if (err && err_len > 0) {
            std::strncpy(err, e.what(), err_len - 1);
            err[err_len - 1] = 0;
        }
        return -1;
    }
}

}  // extern "C"
