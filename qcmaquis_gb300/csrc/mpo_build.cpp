// Two-site MPO tensors on the host, in native code (make_twosite_mpo,
// dmrg/framework/dmrg/mp_tensors/ts_ops.h:78-152).
//
// W(b1,b3) = sum over b2 of W1(b1,b2) (x) W2(b2,b3), one operator per product
// spin s allowed by the bond spins (ts_ops.h:21-35).  The spin-coupled
// Kronecker product of two site operators depends only on the two operators,
// the three bond spins and s, so a tensor needs few distinct products: phase 1
// walks the non-zero (b1, b2, b3) chains and lists them, the caller forms each
// once (the SU(2) op_kron), and phase 2 sums the scaled products of every
// (b1, b3, s) in the reference's order and writes the flattened tensor
// (qcm_mpo_t layout) that the plan builders read.
#include <algorithm>
#include <array>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <vector>

#include "plan.hpp"

using qcm::Q;
using qcm::set_error;

struct qcm_mpo_buf {
    int32_t row_dim = 0, col_dim = 0, symmetry = QCM_SYM_SU2U1;
    std::vector<int32_t> left_spin, right_spin, left_herm, right_herm, left_phase, right_phase;
    // phase 1: distinct products (op1, op2, j, jpp, jp, s) and, per output operator
    // in the reference's table order (b1, b3 ascending, s ascending), its summands
    std::vector<int32_t> keys;
    struct Out { int32_t b1, b3, s; int64_t sb, se; };
    std::vector<Out> outs;
    std::vector<int32_t> sum_prod;
    std::vector<double> sum_coeff;
    // phase 2: the flattened tensor
    bool built = false;
    std::vector<int32_t> col_ptr, row_of, term_ptr, term_op, op_spin, op_blk_ptr, blk_q, blk_ent_ptr, ent, term_pos;
    std::vector<double> term_scale, ent_coeff;
};

namespace {

struct KeyHash {
    size_t operator()(const std::array<int32_t, 6>& k) const {
        uint64_t h = 1469598103934665603ull;
        for (int32_t x : k) { h ^= (uint32_t)x; h *= 1099511628211ull; }
        return (size_t)h;
    }
};

// Operator tables of a flattened MPO (or of a product list): non-null arrays,
// monotone block and entry pointers starting at 0.
void check_ops(const qcm_mpo_t* w, const char* what) {
    if (w->n_ops < 0 || (w->n_ops > 0 && (!w->op_blk_ptr || !w->blk_q || !w->blk_ent_ptr)))
        throw std::runtime_error(std::string("malformed operator tables of ") + what);
    if (w->n_ops == 0) return;
    if (w->op_blk_ptr[0] != 0) throw std::runtime_error(std::string("op_blk_ptr[0] != 0 in ") + what);
    for (int32_t o = 0; o < w->n_ops; ++o)
        if (w->op_blk_ptr[o + 1] < w->op_blk_ptr[o])
            throw std::runtime_error(std::string("op_blk_ptr not monotone in ") + what);
    const int32_t nblk = w->op_blk_ptr[w->n_ops];
    if (w->blk_ent_ptr[0] != 0) throw std::runtime_error(std::string("blk_ent_ptr[0] != 0 in ") + what);
    for (int32_t k = 0; k < nblk; ++k)
        if (w->blk_ent_ptr[k + 1] < w->blk_ent_ptr[k])
            throw std::runtime_error(std::string("blk_ent_ptr not monotone in ") + what);
    if (w->blk_ent_ptr[nblk] > 0 && (!w->ent || !w->ent_coeff))
        throw std::runtime_error(std::string("null operator entries in ") + what);
}

void check_mpo(const qcm_mpo_t* w, const char* what) {
    if (!w) throw std::runtime_error(std::string("null ") + what);
    if (w->row_dim < 0 || w->col_dim < 0 || !w->col_ptr || !w->term_ptr || !w->left_spin || !w->right_spin)
        throw std::runtime_error(std::string("malformed ") + what);
    if (w->col_ptr[0] != 0) throw std::runtime_error(std::string("col_ptr[0] != 0 in ") + what);
    for (int32_t b = 0; b < w->col_dim; ++b)
        if (w->col_ptr[b + 1] < w->col_ptr[b]) throw std::runtime_error(std::string("col_ptr not monotone in ") + what);
    int64_t ne = w->col_ptr[w->col_dim];
    if (ne > 0 && (!w->row_of || !w->term_op || !w->term_scale))
        throw std::runtime_error(std::string("null element arrays in ") + what);
    if (w->term_ptr[0] != 0) throw std::runtime_error(std::string("term_ptr[0] != 0 in ") + what);
    for (int64_t e = 0; e < ne; ++e) {
        if (w->row_of[e] < 0 || w->row_of[e] >= w->row_dim) throw std::runtime_error("mpo row index out of range");
        if (w->term_ptr[e + 1] < w->term_ptr[e]) throw std::runtime_error("mpo term_ptr not monotone");
        for (int t = w->term_ptr[e]; t < w->term_ptr[e + 1]; ++t)
            if (w->term_op[t] < 0 || w->term_op[t] >= w->n_ops) throw std::runtime_error("mpo operator out of range");
    }
    if (w->n_ops > 0 && !w->op_spin) throw std::runtime_error(std::string("null op_spin in ") + what);
    if (w->symmetry != QCM_SYM_SU2U1 && w->symmetry != QCM_SYM_TWOU1 && w->symmetry != QCM_SYM_U1)
        throw std::runtime_error(std::string("unknown symmetry in ") + what);
    check_ops(w, what);
}

// rows of a CSC tensor: b1 -> [(b2, element)], b2 ascending
std::vector<std::vector<std::pair<int32_t, int32_t>>> rows_of(const qcm_mpo_t* w) {
    std::vector<std::vector<std::pair<int32_t, int32_t>>> r(w->row_dim);
    for (int b2 = 0; b2 < w->col_dim; ++b2)
        for (int e = w->col_ptr[b2]; e < w->col_ptr[b2 + 1]; ++e) r[w->row_of[e]].push_back({b2, e});
    return r;
}

void phase1(qcm_mpo_buf& B, const qcm_mpo_t* w1, const qcm_mpo_t* w2) {
    if (w1->col_dim != w2->row_dim) throw std::runtime_error("the MPO tensors do not share a bond");
    if (w1->symmetry != w2->symmetry) throw std::runtime_error("the MPO tensors are of different symmetry groups");
    B.symmetry = w1->symmetry;
    B.row_dim = w1->row_dim;
    B.col_dim = w2->col_dim;
    B.left_spin.assign(w1->left_spin, w1->left_spin + w1->row_dim);
    B.right_spin.assign(w2->right_spin, w2->right_spin + w2->col_dim);
    auto copy_or_identity = [](const int32_t* p, int n, bool herm) {
        std::vector<int32_t> v(n);
        for (int i = 0; i < n; ++i) v[i] = p ? p[i] : (herm ? i : 1);
        return v;
    };
    B.left_herm = copy_or_identity(w1->left_herm, w1->row_dim, true);
    B.left_phase = copy_or_identity(w1->left_phase, w1->row_dim, false);
    B.right_herm = copy_or_identity(w2->right_herm, w2->col_dim, true);
    B.right_phase = copy_or_identity(w2->right_phase, w2->col_dim, false);
    auto rows1 = rows_of(w1);
    auto rows2 = rows_of(w2);
    std::unordered_map<std::array<int32_t, 6>, int32_t, KeyHash> kid;
    // b3 -> [(b2, element of W1, element of W2)] for the current b1
    std::vector<std::vector<std::array<int32_t, 3>>> chains(w2->col_dim);
    std::vector<int32_t> touched;
    struct Acc { std::vector<int32_t> prod; std::vector<double> coeff; };
    std::map<int, Acc> per_s;
    for (int b1 = 0; b1 < w1->row_dim; ++b1) {
        touched.clear();
        for (auto& [b2, e1] : rows1[b1])
            for (auto& [b3, e2] : rows2[b2]) {
                if (chains[b3].empty()) touched.push_back(b3);
                chains[b3].push_back({b2, e1, e2});
            }
        std::sort(touched.begin(), touched.end());
        const int j = w1->left_spin[b1];
        for (int b3 : touched) {
            const int jp = w2->right_spin[b3];
            per_s.clear();
            for (auto& ch : chains[b3]) {
                const int jpp = w1->right_spin[ch[0]];
                for (int t1 = w1->term_ptr[ch[1]]; t1 < w1->term_ptr[ch[1] + 1]; ++t1) {
                    const int o1 = w1->term_op[t1], k1 = w1->op_spin[o1];
                    for (int t2 = w2->term_ptr[ch[2]]; t2 < w2->term_ptr[ch[2] + 1]; ++t2) {
                        const int o2 = w2->term_op[t2], k2 = w2->op_spin[o2];
                        for (int s = std::abs(k1 - k2); s <= std::abs(k1 + k2); s += 2) {
                            if (!(std::abs(s - j) <= jp && jp <= std::abs(s + j))) continue;
                            std::array<int32_t, 6> key{o1, o2, j, jpp, jp, s};
                            auto it = kid.find(key);
                            if (it == kid.end()) {
                                it = kid.emplace(key, (int32_t)(B.keys.size() / 6)).first;
                                B.keys.insert(B.keys.end(), key.begin(), key.end());
                            }
                            Acc& a = per_s[s];
                            a.prod.push_back(it->second);
                            a.coeff.push_back(w1->term_scale[t1] * w2->term_scale[t2]);
                        }
                    }
                }
            }
            for (auto& [s, a] : per_s) {
                qcm_mpo_buf::Out o{b1, b3, s, (int64_t)B.sum_prod.size(), 0};
                B.sum_prod.insert(B.sum_prod.end(), a.prod.begin(), a.prod.end());
                B.sum_coeff.insert(B.sum_coeff.end(), a.coeff.begin(), a.coeff.end());
                o.se = (int64_t)B.sum_prod.size();
                B.outs.push_back(o);
            }
            chains[b3].clear();
        }
    }
}

struct Entry { int32_t r, c, rs, cs; double v; };
// entries in first-occurrence order; pos maps (row, col) to the entry, so each
// summand is found in constant time and the summation order is unchanged
struct Block {
    Q lc, rc;
    std::vector<Entry> e;
    std::unordered_map<uint64_t, int32_t> pos;
};
inline uint64_t rc_key(int32_t r, int32_t c) { return ((uint64_t)(uint32_t)r << 32) | (uint32_t)c; }

void phase2(qcm_mpo_buf& B, const qcm_mpo_t* prods) {
    const int64_t nkeys = (int64_t)B.keys.size() / 6;
    if (!prods || prods->n_ops != nkeys || !prods->op_blk_ptr || !prods->blk_q || !prods->blk_ent_ptr)
        throw std::runtime_error("one product operator per listed key expected");
    check_ops(prods, "the product operators");
    // start from empty output tables, so a retry after a failed finish rebuilds cleanly
    B.built = false;
    B.col_ptr.clear(); B.row_of.clear(); B.term_ptr.clear(); B.term_op.clear(); B.op_spin.clear();
    B.op_blk_ptr.clear(); B.blk_q.clear(); B.blk_ent_ptr.clear(); B.ent.clear(); B.term_pos.clear();
    B.term_scale.clear(); B.ent_coeff.clear();
    // the output operators, grouped per element (b1, b3) in column-major order;
    // an element lists its operators with s descending (later table entries first)
    std::vector<int64_t> order(B.outs.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int64_t)i;
    std::stable_sort(order.begin(), order.end(), [&](int64_t a, int64_t b) {
        const auto &x = B.outs[a], &y = B.outs[b];
        if (x.b3 != y.b3) return x.b3 < y.b3;
        return x.b1 < y.b1;
    });
    B.col_ptr.assign(1, 0);
    B.term_ptr.assign(1, 0);
    B.op_blk_ptr.assign(1, 0);
    B.blk_ent_ptr.assign(1, 0);
    std::vector<Block> blocks;
    size_t i = 0;
    for (int b3 = 0; b3 < B.col_dim; ++b3) {
        while (i < order.size() && B.outs[order[i]].b3 == b3) {
            size_t k = i;
            const int b1 = B.outs[order[i]].b1;
            while (k < order.size() && B.outs[order[k]].b3 == b3 && B.outs[order[k]].b1 == b1) ++k;
            B.row_of.push_back(b1);
            for (size_t q = k; q-- > i;) {   // s descending
                const auto& o = B.outs[order[q]];
                B.term_pos.push_back((int32_t)(k - 1 - q));
                B.term_op.push_back((int32_t)B.op_spin.size());
                B.term_scale.push_back(1.0);
                B.op_spin.push_back(o.s);
                // sum of the scaled products, summand by summand, entry by entry
                blocks.clear();
                for (int64_t t = o.sb; t < o.se; ++t) {
                    const int p = B.sum_prod[t];
                    const double c = B.sum_coeff[t];
                    for (int kb = prods->op_blk_ptr[p]; kb < prods->op_blk_ptr[p + 1]; ++kb) {
                        Q lc(prods->blk_q[4 * kb], prods->blk_q[4 * kb + 1]);
                        Q rc(prods->blk_q[4 * kb + 2], prods->blk_q[4 * kb + 3]);
                        Block* bl = nullptr;
                        for (auto& x : blocks)
                            if (x.lc == lc && x.rc == rc) { bl = &x; break; }
                        if (!bl) { blocks.push_back({lc, rc, {}, {}}); bl = &blocks.back(); }
                        for (int en = prods->blk_ent_ptr[kb]; en < prods->blk_ent_ptr[kb + 1]; ++en) {
                            const int32_t* x = prods->ent + 4 * en;
                            const double v = prods->ent_coeff[en] * c;
                            auto it = bl->pos.find(rc_key(x[0], x[1]));
                            if (it != bl->pos.end()) {
                                Entry& y = bl->e[it->second];
                                y.v = y.v + v;
                            } else {
                                bl->pos.emplace(rc_key(x[0], x[1]), (int32_t)bl->e.size());
                                bl->e.push_back({x[0], x[1], x[2], x[3], v});
                            }
                        }
                    }
                }
                std::sort(blocks.begin(), blocks.end(), [](const Block& a, const Block& b) {
                    return a.lc > b.lc || (a.lc == b.lc && a.rc > b.rc);
                });
                for (auto& bl : blocks) {
                    B.blk_q.insert(B.blk_q.end(), {bl.lc.n, bl.lc.s, bl.rc.n, bl.rc.s});
                    std::sort(bl.e.begin(), bl.e.end(), [](const Entry& a, const Entry& b) {
                        return a.r < b.r || (a.r == b.r && a.c < b.c);
                    });
                    for (auto& y : bl.e) {
                        if (y.v == 0.0) continue;
                        B.ent.insert(B.ent.end(), {y.r, y.c, y.rs, y.cs});
                        B.ent_coeff.push_back(y.v);
                    }
                    B.blk_ent_ptr.push_back((int32_t)B.ent_coeff.size());
                }
                B.op_blk_ptr.push_back((int32_t)B.blk_ent_ptr.size() - 1);
            }
            B.term_ptr.push_back((int32_t)B.term_op.size());
            i = k;
        }
        B.col_ptr.push_back((int32_t)B.row_of.size());
    }
    if (B.ent_coeff.size() > (size_t)INT32_MAX || B.term_op.size() > (size_t)INT32_MAX)
        throw std::runtime_error("two-site tensor too large for 32-bit offsets");
    B.built = true;
}

// The operators of a flattened tensor's products, in the qcm_mpo_t operator layout.
struct ProdOps {
    std::vector<int32_t> op_spin, op_blk_ptr{0}, blk_q, blk_ent_ptr{0}, ent;
    std::vector<double> ent_coeff;
    qcm_mpo_t view() const {
        qcm_mpo_t v;
        std::memset(&v, 0, sizeof(v));
        v.n_ops = (int32_t)op_spin.size();
        v.op_spin = op_spin.data();
        v.op_blk_ptr = op_blk_ptr.data();
        v.blk_q = blk_q.data();
        v.blk_ent_ptr = blk_ent_ptr.data();
        v.ent = ent.data();
        v.ent_coeff = ent_coeff.data();
        return v;
    }
};

struct DenseBlock { Q in, out; int64_t rows, cols; std::vector<double> v; };  // row-major

std::vector<DenseBlock> dense_op(const qcm_mpo_t* w, int o, const qcm::Idx& phys) {
    std::vector<DenseBlock> r;
    for (int kb = w->op_blk_ptr[o]; kb < w->op_blk_ptr[o + 1]; ++kb) {
        DenseBlock b;
        b.in = Q(w->blk_q[4 * kb], w->blk_q[4 * kb + 1]);
        b.out = Q(w->blk_q[4 * kb + 2], w->blk_q[4 * kb + 3]);
        b.rows = phys.size_of(b.in);
        b.cols = phys.size_of(b.out);
        b.v.assign((size_t)(b.rows * b.cols), 0.0);
        for (int en = w->blk_ent_ptr[kb]; en < w->blk_ent_ptr[kb + 1]; ++en) {
            const int r0 = w->ent[4 * en], c0 = w->ent[4 * en + 1];
            if (r0 < 0 || r0 >= b.rows || c0 < 0 || c0 >= b.cols) throw std::runtime_error("operator entry outside its block");
            b.v[(size_t)(r0 * b.cols + c0)] = w->ent_coeff[en];
        }
        r.push_back(std::move(b));
    }
    return r;
}

// The small identity of a spin-0 operator next to a spin > 0 one is extended by the
// two off-diagonal unit entries between the second and third local charges
// (site_operator_algorithms.h:238-256).
void expand_identity(std::vector<DenseBlock>& op, const qcm::Idx& phys) {
    if (phys.size() < 3) return;
    const Q cb = phys.d[1].first, cc = phys.d[2].first;
    for (auto& b : op)
        if (b.in == cb && b.out == cc) return;
    op.push_back({cb, cc, 1, 1, {1.0}});
    op.push_back({cc, cb, 1, 1, {1.0}});
}

int product_spin(Q a, Q b) { return (a.s == -1 && b.s == 1) ? 2 : std::abs(a.s + b.s); }

double mod_coupling9(int a, int b, int c, int d, int e, int f, int g, int h, int i) {
    return std::sqrt((g + 1.0) * (h + 1.0) * (c + 1.0) * (f + 1.0)) * qcm::wigner9j(a, b, c, d, e, f, g, h, i);
}

// op_kron for SU(2) (site_operator_algorithms.h): the spin-coupled Kronecker product
// of operator o1 of W1 and o2 of W2 for bond spins (j, jpp, jp) and product spin k.
// For an abelian group (abelian = true) the plain Kronecker product
// (site_operator_algorithms.h:167-205): no identity expansion, couplings 1.
void op_kron(const qcm_mpo_t* w1, const qcm_mpo_t* w2, int o1, int o2, int j, int jpp, int jp, int k,
             const qcm::Idx& p1, const qcm::Idx& p2, const qcm::PB& pb, ProdOps& out, bool abelian) {
    std::vector<DenseBlock> A = dense_op(w1, o1, p1), Bo = dense_op(w2, o2, p2);
    const int k1 = w1->op_spin[o1], k2 = w2->op_spin[o2];
    if (!abelian && k1 > 0 && k2 == 0) expand_identity(Bo, p2);
    if (!abelian && k1 == 0 && k2 > 0) expand_identity(A, p1);
    struct Acc { int64_t rows, cols; std::vector<double> v; std::vector<int32_t> rs, cs; };
    std::map<std::pair<Q, Q>, Acc, std::function<bool(const std::pair<Q, Q>&, const std::pair<Q, Q>&)>> blocks(
        [](const std::pair<Q, Q>& x, const std::pair<Q, Q>& y) {
            return x.first > y.first || (x.first == y.first && x.second > y.second);   // DualIndex order
        });
    for (const DenseBlock& a : A)
        for (const DenseBlock& b : Bo) {
            const Q nl = qcm::fuse(a.in, b.in), nr = qcm::fuse(a.out, b.out);
            auto it = blocks.find({nl, nr});
            if (it == blocks.end()) {
                Acc z;
                z.rows = pb.size(nl);
                z.cols = pb.size(nr);
                z.v.assign((size_t)(z.rows * z.cols), 0.0);
                z.rs.assign((size_t)z.rows, 0);
                z.cs.assign((size_t)z.cols, 0);
                it = blocks.emplace(std::make_pair(nl, nr), std::move(z)).first;
            }
            Acc& t = it->second;
            const int64_t io = pb(a.in, b.in), oo = pb(a.out, b.out);
            const int J = abelian ? 0 : product_spin(a.in, b.in), Jp = abelian ? 0 : product_spin(a.out, b.out);
            const double c9 = abelian ? 1.0
                                      : mod_coupling9(std::abs(a.in.s), std::abs(b.in.s), J, k1, k2, k,
                                                      std::abs(a.out.s), std::abs(b.out.s), Jp);
            for (int64_t l1 = 0; l1 < a.rows; ++l1)
                for (int64_t r1 = 0; r1 < a.cols; ++r1)
                    for (int64_t l2 = 0; l2 < b.rows; ++l2)
                        for (int64_t r2 = 0; r2 < b.cols; ++r2) {
                            const int64_t row = io + l1 * b.rows + l2, col = oo + r1 * b.cols + r2;
                            t.v[(size_t)(row * t.cols + col)] = (b.v[(size_t)(l2 * b.cols + r2)] *
                                                                 a.v[(size_t)(l1 * a.cols + r1)]) * c9;
                        }
            t.rs[(size_t)io] = J;
            t.cs[(size_t)oo] = Jp;
        }
    double c6 = abelian ? 1.0 : std::sqrt((jpp + 1.0) * (k + 1.0)) * qcm::wigner6j(j, jp, k, k2, k1, jpp);
    if (!abelian && ((j + jp + k1 + k2) / 2) % 2) c6 = -c6;
    out.op_spin.push_back(k);
    for (auto& [key, t] : blocks) {
        bool any = false;
        for (double& x : t.v) {
            x = x * c6;
            if (x != 0.0) any = true;
        }
        if (!any) continue;   // remove_empty_blocks
        out.blk_q.insert(out.blk_q.end(), {key.first.n, key.first.s, key.second.n, key.second.s});
        for (int64_t r0 = 0; r0 < t.rows; ++r0)
            for (int64_t c0 = 0; c0 < t.cols; ++c0) {
                const double x = t.v[(size_t)(r0 * t.cols + c0)];
                if (x == 0.0) continue;
                out.ent.insert(out.ent.end(), {(int32_t)r0, (int32_t)c0, t.rs[(size_t)r0], t.cs[(size_t)c0]});
                out.ent_coeff.push_back(x);
            }
        out.blk_ent_ptr.push_back((int32_t)out.ent_coeff.size());
    }
    out.op_blk_ptr.push_back((int32_t)out.blk_ent_ptr.size() - 1);
}

qcm::Idx read_idx(const qcm_index_t* x) {
    qcm::Idx r;
    if (!x) throw std::runtime_error("null index");
    for (int i = 0; i < x->n; ++i) r.d.push_back({Q(x->q[2 * i], x->q[2 * i + 1]), x->size[i]});
    for (size_t i = 1; i < r.d.size(); ++i)
        if (!(r.d[i - 1].first > r.d[i].first)) throw std::runtime_error("index not sorted descending");
    return r;
}

}  // namespace

extern "C" {

int qcm_mpo_twosite_begin(const qcm_mpo_t* w1, const qcm_mpo_t* w2, qcm_mpo_buf** out, int32_t* n_keys) {
    if (!out || !n_keys) { set_error("qcm_mpo_twosite_begin: null output"); return QCM_E_INVALID; }
    *out = nullptr;
    auto* B = new qcm_mpo_buf();
    try {
        check_mpo(w1, "left MPO tensor");
        check_mpo(w2, "right MPO tensor");
        phase1(*B, w1, w2);
        *n_keys = (int32_t)(B->keys.size() / 6);
        *out = B;
        return QCM_OK;
    } catch (const std::exception& e) {
        delete B;
        set_error(std::string("qcm_mpo_twosite_begin: ") + e.what());
        return QCM_E_INVALID;
    }
}

int qcm_mpo_twosite_keys(const qcm_mpo_buf* B, int32_t* keys) {
    if (!B || !keys) { set_error("qcm_mpo_twosite_keys: null argument"); return QCM_E_INVALID; }
    std::memcpy(keys, B->keys.data(), B->keys.size() * sizeof(int32_t));
    return QCM_OK;
}

int qcm_mpo_twosite_finish(qcm_mpo_buf* B, const qcm_mpo_t* products) {
    if (!B) { set_error("qcm_mpo_twosite_finish: null handle"); return QCM_E_INVALID; }
    try {
        phase2(*B, products);
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_mpo_twosite_finish: ") + e.what());
        return QCM_E_INVALID;
    }
}

int qcm_mpo_buf_view(const qcm_mpo_buf* B, qcm_mpo_t* view, int64_t* sizes) {
    if (!B || !view || !sizes) { set_error("qcm_mpo_buf_view: null argument"); return QCM_E_INVALID; }
    if (!B->built) { set_error("qcm_mpo_buf_view: tensor not built (qcm_mpo_twosite_finish)"); return QCM_E_INVALID; }
    view->row_dim = B->row_dim;
    view->col_dim = B->col_dim;
    view->left_spin = B->left_spin.data();
    view->right_spin = B->right_spin.data();
    view->left_herm = B->left_herm.data();
    view->right_herm = B->right_herm.data();
    view->left_phase = B->left_phase.data();
    view->right_phase = B->right_phase.data();
    view->col_ptr = B->col_ptr.data();
    view->row_of = B->row_of.data();
    view->term_ptr = B->term_ptr.data();
    view->term_op = B->term_op.data();
    view->term_scale = B->term_scale.data();
    view->n_ops = (int32_t)B->op_spin.size();
    view->op_spin = B->op_spin.data();
    view->op_blk_ptr = B->op_blk_ptr.data();
    view->blk_q = B->blk_q.data();
    view->blk_ent_ptr = B->blk_ent_ptr.data();
    view->ent = B->ent.data();
    view->ent_coeff = B->ent_coeff.data();
    view->symmetry = B->symmetry;
    sizes[0] = (int64_t)B->row_of.size();        // elements
    sizes[1] = (int64_t)B->term_op.size();       // terms (= operators)
    sizes[2] = (int64_t)B->blk_q.size() / 4;     // operator blocks
    sizes[3] = (int64_t)B->ent_coeff.size();     // entries
    return QCM_OK;
}

int qcm_mpo_buf_term_pos(const qcm_mpo_buf* B, int32_t* pos) {
    if (!B || !pos || !B->built) { set_error("qcm_mpo_buf_term_pos: no built tensor"); return QCM_E_INVALID; }
    std::memcpy(pos, B->term_pos.data(), B->term_pos.size() * sizeof(int32_t));
    return QCM_OK;
}

int qcm_mpo_twosite(const qcm_mpo_t* w1, const qcm_mpo_t* w2, const qcm_index_t* phys1, const qcm_index_t* phys2,
                    qcm_mpo_buf** out) {
    if (!out) { set_error("qcm_mpo_twosite: null output"); return QCM_E_INVALID; }
    *out = nullptr;
    auto* B = new qcm_mpo_buf();
    try {
        check_mpo(w1, "left MPO tensor");
        check_mpo(w2, "right MPO tensor");
        const qcm::Idx p1 = read_idx(phys1), p2 = read_idx(phys2);
        const qcm::PB pb(p1, p2, false);
        phase1(*B, w1, w2);
        ProdOps prods;
        for (size_t q = 0; q + 5 < B->keys.size(); q += 6) {
            const int32_t* k = &B->keys[q];
            op_kron(w1, w2, k[0], k[1], k[2], k[3], k[4], k[5], p1, p2, pb, prods, w1->symmetry != QCM_SYM_SU2U1);
        }
        const qcm_mpo_t v = prods.view();
        phase2(*B, &v);
        *out = B;
        return QCM_OK;
    } catch (const std::exception& e) {
        delete B;
        set_error(std::string("qcm_mpo_twosite: ") + e.what());
        return QCM_E_INVALID;
    }
}

void qcm_mpo_buf_destroy(qcm_mpo_buf* B) { delete B; }

}  // extern "C"
