// Terms of the SU2U1 quantum-chemistry Hamiltonian from its integrals, in native
// code (qc_su2 model, dmrg/framework/dmrg/models/chem/su2u1/model.hpp:52-203, with
// the SU(2) term makers of models/chem/su2u1/term_maker.h:120-395 and the spin
// sums of models/chem/su2u1/chem_helper.h / term_maker.h:548-793).
//
// Every integral (i, j, k, l) becomes its operator terms: one-site terms (core
// energy, number and double-occupancy operators) kept as they come, two-, three-
// and four-operator terms merged with equal terms (same positions and operators)
// by summing their coefficients.  Off-diagonal one-body integrals are folded into
// two-body terms with weight 1/(N-1) (model.hpp:96-139).  Each term records its
// coefficient as a combination of the integral values: per integral, the
// coefficient that one unit of it contributes (the energy gradient reads these).
// Output order: the one-site terms in integral order, then the merged two-,
// three- and four-operator terms, each in ascending order of (positions, tags).
#include <algorithm>
#include <cmath>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "plan.hpp"

using qcm::set_error;

namespace {

enum BundleId { B_CREATE, B_DESTROY, B_COUNT, B_FLIP, B_E2D, B_D2E, B_DOCC, B_CREATE_COUNT, B_DESTROY_COUNT };
enum Field { COUPLE_UP, COUPLE_DOWN, FILL_COUPLE_UP, FILL_COUPLE_DOWN, NO_COUPLE, FILL_NO_COUPLE };

struct Op { int32_t pos, tag; };
struct Term {
    std::vector<Op> ops;
    double coeff = 0.0;
    bool ferm = false;
    std::vector<std::pair<int64_t, double>> src;   // (integral index, coefficient per unit), insertion order
};

bool sgn4(int i, int j, int k, int l) {
    const int idx[4] = {i, j, k, l};
    int inv = 0;
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 4; ++b)
            if (idx[a] > idx[b]) ++inv;
    return inv % 2 != 0;
}

void align(int& i, int& j, int& k, int& l) {   // canonical order, models/chem/util.h:97-110
    if (i < j) std::swap(i, j);
    if (k < l) std::swap(k, l);
    if (i < k) { std::swap(i, k); std::swap(j, l); }
    if (i == k && j < l) std::swap(j, l);
}

struct Gen {
    const qcm_chem_tags_t& t;
    int L, N;

    int32_t tag(int b, int f) const {
        const int32_t x = t.bundles[b][f];
        if (x < 0) throw std::runtime_error("operator missing from the tag table");
        return x;
    }

    // term_maker two_term / positional_two_term / three_term / four_term
    Term two(bool sign, double scale, int i, int j, int32_t op1, int32_t op2) const {
        Term r;
        r.coeff = scale;
        r.ferm = sign;
        r.ops = {{i, op1}, {j, op2}};
        return r;
    }
    Term positional_two(bool sign, double scale, int i, int j, int32_t op1, int32_t op1_fill, int32_t op2,
                        int32_t op2_fill) const {
        Term r;
        r.coeff = scale;
        r.ferm = sign;
        const int32_t op1_use = i < j ? op1_fill : op2_fill;
        const int32_t op2_use = i < j ? op2 : op1;
        if (j < i && sign) r.coeff = -r.coeff;
        r.ops = {{std::min(i, j), op1_use}, {std::max(i, j), op2_use}};
        return r;
    }
    Term three(double scale, int pb, int p1, int p2, int32_t boson, int32_t boson_fill, int32_t op1, int32_t op1_fill,
               int32_t op2, int32_t op2_fill) const {
        Term r;
        r.coeff = scale;
        r.ferm = true;
        const int32_t op1_use = p1 < p2 ? op1_fill : op2_fill;
        const int32_t op2_use = p1 < p2 ? op2 : op1;
        const int32_t boson_use = ((p1 < pb && pb < p2) || (p2 < pb && pb < p1)) ? boson_fill : boson;
        if (p2 < p1) r.coeff = -r.coeff;
        r.ops = {{pb, boson_use}, {std::min(p1, p2), op1_use}, {std::max(p1, p2), op2_use}};
        std::stable_sort(r.ops.begin(), r.ops.end(), [](const Op& a, const Op& b) { return a.pos < b.pos; });
        return r;
    }
    Term four(int max_two_S, double scale, int i, int j, int k, int l, int bi, int bk) const {
        Term r;
        r.coeff = scale;
        r.ferm = true;
        if (sgn4(i, j, k, l)) r.coeff = -r.coeff;
        std::pair<int, int> st[4] = {{i, bi}, {j, bi}, {k, bk}, {l, bk}};
        std::stable_sort(st, st + 4, [](const auto& a, const auto& b) { return a.first < b.first; });
        const int f[4] = {FILL_COUPLE_UP, max_two_S == 2 ? COUPLE_UP : COUPLE_DOWN,
                          max_two_S == 2 ? FILL_COUPLE_DOWN : FILL_COUPLE_UP, COUPLE_DOWN};
        for (int q = 0; q < 4; ++q) r.ops.push_back({st[q].first, tag(st[q].second, f[q])});
        return r;
    }

    // SpinSumSU2
    void V_term(double me, int i, int k, int l, int j, std::vector<Term>& out) const {
        int u[4] = {i, k, l, j};
        std::sort(u, u + 4);
        const int n_unique = (int)(std::unique(u, u + 4) - u);
        if (n_unique == 4) return four_term(me, i, k, l, j, out);
        if (n_unique == 3) return three_term(me, i, k, l, j, out);
        if (n_unique == 2) return two_term(me, i, k, l, j, out);
        Term r;
        r.coeff = 2.0 * me;
        r.ops = {{i, tag(B_DOCC, NO_COUPLE)}};
        out.push_back(r);
    }

    void two_term(double me, int i, int k, int l, int j, std::vector<Term>& out) const {
        const int32_t count = tag(B_COUNT, NO_COUPLE);
        if (i == j && k == l && j != k) {
            out.push_back(two(false, me, i, k, count, count));
            return;
        }
        if (i == k && j == l && j != k) {
            out.push_back(two(false, 2.0 * me, i, j, tag(B_E2D, NO_COUPLE), tag(B_D2E, NO_COUPLE)));
            return;
        }
        if (i == l && j == k && i != j) {
            out.push_back(positional_two(false, std::sqrt(3.0) * me, i, j, tag(B_FLIP, COUPLE_DOWN),
                                         tag(B_FLIP, COUPLE_UP), tag(B_FLIP, COUPLE_DOWN), tag(B_FLIP, COUPLE_UP)));
            out.push_back(two(false, -0.5 * me, i, j, count, count));
            return;
        }
        if ((i == k && k == l) || (k == l && l == j) || (i == l && l == j) || (i == k && k == j)) {
            int s, p;
            if (i == k && k == l) { s = i; p = j; }
            else if (k == l && l == j) { s = j; p = i; }
            else if (i == l && l == j) { s = i; p = k; }
            else { s = i; p = l; }
            if (i == k)
                out.push_back(positional_two(true, std::sqrt(2.0) * me, s, p, tag(B_CREATE_COUNT, COUPLE_DOWN),
                                             tag(B_CREATE_COUNT, FILL_COUPLE_UP), tag(B_DESTROY, COUPLE_DOWN),
                                             tag(B_DESTROY, FILL_COUPLE_UP)));
            else
                out.push_back(positional_two(true, -std::sqrt(2.0) * me, s, p, tag(B_DESTROY_COUNT, COUPLE_DOWN),
                                             tag(B_DESTROY_COUNT, FILL_COUPLE_UP), tag(B_CREATE, COUPLE_DOWN),
                                             tag(B_CREATE, FILL_COUPLE_UP)));
            return;
        }
        throw std::runtime_error("unexpected index arrangement for a V_ijjj term");
    }

    void three_term(double me, int i, int k, int l, int j, std::vector<Term>& out) const {
        if (i == j || k == l) return three_termA(me, i, k, l, j, out);
        three_termB(me, i, k, l, j, out);
    }

    void four_term(double me, int i, int k, int l, int j, std::vector<Term>& out) const {
        int i_ = i, j_ = j, k_ = k, l_ = l;
        align(i_, j_, k_, l_);
        if (k_ > l_ && l_ > j_) {
            out.push_back(four(2, -std::sqrt(3.0) * me, i, k, l, j, B_CREATE, B_DESTROY));
            out.push_back(four(1, me, i, k, l, j, B_CREATE, B_DESTROY));
        } else if (k_ > j_ && j_ > l_) {
            const double le = sgn4(i, k, l, j) ? -me : me;
            out.push_back(four(2, std::sqrt(3.0) * le, i, k, l, j, B_CREATE, B_DESTROY));
            out.push_back(four(1, le, i, k, l, j, B_CREATE, B_DESTROY));
        } else if (j_ > k_ && k_ > l_) {
            out.push_back(four(1, 2.0 * me, i, k, l, j, B_CREATE, B_DESTROY));
        } else {
            throw std::runtime_error("unexpected index arrangement in a V_ijkl term");
        }
    }

    void three_termA(double me, int i, int k, int l, int j, std::vector<Term>& out) const {
        int same = -1;
        if (i == j) same = i;
        if (k == l) { same = k; k = i; l = j; }
        out.push_back(three(std::sqrt(2.0) * me, same, k, l, tag(B_COUNT, NO_COUPLE), tag(B_COUNT, FILL_NO_COUPLE),
                            tag(B_CREATE, COUPLE_DOWN), tag(B_CREATE, FILL_COUPLE_UP), tag(B_DESTROY, COUPLE_DOWN),
                            tag(B_DESTROY, FILL_COUPLE_UP)));
    }

    void three_termB(double me, int i, int k, int l, int j, std::vector<Term>& out) const {
        const int32_t cd = tag(B_CREATE, COUPLE_DOWN), cfu = tag(B_CREATE, FILL_COUPLE_UP);
        const int32_t dd = tag(B_DESTROY, COUPLE_DOWN), dfu = tag(B_DESTROY, FILL_COUPLE_UP);
        const int32_t count = tag(B_COUNT, NO_COUPLE);
        if (i == k) {
            const int32_t e2d = tag(B_E2D, NO_COUPLE);
            out.push_back(three(-std::sqrt(2.0) * me, i, std::min(l, j), std::max(l, j), e2d, e2d, dd, dfu, dd, dfu));
        }
        if (j == l) {
            const int32_t d2e = tag(B_D2E, NO_COUPLE);
            out.push_back(three(-std::sqrt(2.0) * me, j, std::min(i, k), std::max(i, k), d2e, d2e, cd, cfu, cd, cfu));
        }
        if (j == k || i == l) {
            int same, p1, p2;
            if (j == k) { same = j; p1 = l; p2 = i; }
            else { same = i; p1 = j; p2 = k; }
            const double phase = sgn4(i, k, l, j) ? -1.0 : 1.0;
            if (same < std::min(p1, p2)) {
                const int32_t fu = tag(B_FLIP, COUPLE_UP);
                out.push_back(three(phase * std::sqrt(3.0) * me, same, p1, p2, fu, fu, cd,
                                    tag(B_CREATE, FILL_COUPLE_DOWN), dd, tag(B_DESTROY, FILL_COUPLE_DOWN)));
                out.push_back(three(-0.5 * std::sqrt(2.0) * me, same, p1, p2, count, count, cd, cfu, dd, dfu));
            } else if (same > std::max(p1, p2)) {
                const int32_t fd = tag(B_FLIP, COUPLE_DOWN);
                out.push_back(three(phase * std::sqrt(3.0) * me, same, p1, p2, fd, fd, tag(B_CREATE, COUPLE_UP), cfu,
                                    tag(B_DESTROY, COUPLE_UP), dfu));
                out.push_back(three(-0.5 * std::sqrt(2.0) * me, same, p1, p2, count, count, cd, cfu, dd, dfu));
            } else {
                const int32_t fn = tag(B_FLIP, NO_COUPLE), cfn = tag(B_COUNT, FILL_NO_COUPLE);
                out.push_back(three(phase * std::sqrt(3.0) * me, same, p1, p2, fn, fn, cd, cfu, dd, dfu));
                out.push_back(three(-0.5 * std::sqrt(2.0) * me, same, p1, p2, cfn, cfn, cd, cfu, dd, dfu));
            }
        }
    }

    // the terms of one integral as (kind, term): kind 1 = kept as is, 2/3/4 = merged
    void integral_terms(int i, int j, int k, int l, double me, std::vector<std::pair<int, Term>>& out) const {
        std::vector<Term> ts;
        auto take = [&](int kind) {
            for (auto& x : ts) out.push_back({kind, std::move(x)});
            ts.clear();
        };
        if (i == -1 && j == -1 && k == -1 && l == -1) {
            Term r;
            r.coeff = me;
            r.ops = {{0, t.ident}};
            out.push_back({1, r});
        } else if (i == j && k == -1 && l == -1) {
            Term r;
            r.coeff = me;
            r.ops = {{i, t.count}};
            out.push_back({1, r});
        } else if (k == -1 && l == -1) {
            if (N == 1) throw std::runtime_error("one-electron systems are not supported");
            const double f = me * (1.0 / (N - 1));
            for (int kk = 0; kk < L; ++kk) {
                if (kk == j || kk == i) continue;
                three_term(f, i, kk, kk, j, ts);
                three_term(f, j, kk, kk, i, ts);
            }
            take(3);
            V_term(f, i, i, i, j, ts);
            V_term(f, j, i, i, i, ts);
            V_term(f, i, j, j, j, ts);
            V_term(f, j, j, j, i, ts);
            take(2);
        } else if (i == j && j == k && k == l) {
            Term r;
            r.coeff = me;
            r.ops = {{i, t.docc}};
            out.push_back({1, r});
        } else if ((i == j && j == k && k != l) || (i != j && j == k && k == l)) {
            int s, p;
            if (i == j) { s = i; p = l; }
            else if (k == l) { s = l; p = i; }
            else throw std::runtime_error("V_ijjj");
            two_term(me, s, s, s, p, ts);
            two_term(me, s, p, s, s, ts);
            take(2);
        } else if (i == j && k == l && j != k) {
            two_term(me, i, k, k, i, ts);
            take(2);
        } else if (i == k && j == l && i != j) {
            two_term(0.5 * me, i, i, j, j, ts);
            two_term(0.5 * me, j, j, i, i, ts);
            two_term(me, i, j, i, j, ts);
            take(2);
        } else if ((i == j && j != k && k != l) || (k == l && i != j && j != k)) {
            if (i == j) {
                three_term(me, i, k, l, i, ts);
                three_term(me, i, l, k, i, ts);
            } else {
                three_term(me, i, k, k, j, ts);
                three_term(me, j, k, k, i, ts);
            }
            take(3);
        } else if (((i == k && j != l) || j == k || (j == l && i != k)) && (i != j && k != l)) {
            three_term(me, i, k, l, j, ts);
            three_term(me, i, l, k, j, ts);
            three_term(me, j, k, l, i, ts);
            three_term(me, j, l, k, i, ts);
            take(3);
        } else if (i != j && j != k && k != l && i != k && j != l) {
            four_term(me, i, k, l, j, ts);
            four_term(me, i, l, k, j, ts);
            four_term(me, j, k, l, i, ts);
            four_term(me, j, l, k, i, ts);
            take(4);
        }
    }
};

}  // namespace

struct qcm_term_buf {
    std::vector<int32_t> term_ptr{0}, pos, tag, ferm;
    std::vector<double> coeff;
    std::vector<int64_t> src_ptr{0}, src_idx;
    std::vector<double> src_val;
};

extern "C" {

int qcm_chem_terms(int32_t L, int32_t nelec, int64_t n_int, const int32_t* idx, const double* val, double cutoff,
                   const qcm_chem_tags_t* tags, qcm_term_buf** out) {
    if (!out) { set_error("qcm_chem_terms: null output"); return QCM_E_INVALID; }
    *out = nullptr;
    if (!tags || L <= 0 || n_int < 0 || (n_int > 0 && (!idx || !val))) {
        set_error("qcm_chem_terms: invalid argument");
        return QCM_E_INVALID;
    }
    auto* B = new qcm_term_buf();
    try {
        Gen g{*tags, L, nelec};
        std::vector<Term> one_site;
        std::map<std::vector<int32_t>, Term> merged[3];   // two-, three-, four-operator terms by key
        std::vector<std::pair<int, Term>> ts, units;
        for (int64_t q = 0; q < n_int; ++q) {
            const double me = val[q];
            if (!(std::fabs(me) > cutoff)) continue;
            int i = idx[4 * q] - 1, j = idx[4 * q + 1] - 1, k = idx[4 * q + 2] - 1, l = idx[4 * q + 3] - 1;
            for (int x : {i, j, k, l})
                if (x < -1 || x >= L) throw std::runtime_error("integral index out of range");
            align(i, j, k, l);
            ts.clear();
            g.integral_terms(i, j, k, l, me, ts);
            if (me == 0.0) {   // the coefficient per unit of an integral of value zero
                units.clear();
                g.integral_terms(i, j, k, l, 1.0, units);
            }
            for (size_t a = 0; a < ts.size(); ++a) {
                Term& t = ts[a].second;
                t.src = {{q, me != 0.0 ? t.coeff / me : units[a].second.coeff}};
                const int kind = ts[a].first;
                if (kind == 1) {
                    one_site.push_back(std::move(t));
                    continue;
                }
                std::vector<int32_t> key;
                for (const Op& o : t.ops) key.push_back(o.pos);
                for (const Op& o : t.ops) key.push_back(o.tag);
                auto& store = merged[kind - 2];
                auto it = store.find(key);
                if (it == store.end()) {
                    store.emplace(std::move(key), std::move(t));
                } else {
                    Term& m = it->second;
                    m.coeff += t.coeff;
                    for (const auto& s : t.src) {
                        auto sit = std::find_if(m.src.begin(), m.src.end(),
                                                [&](const auto& x) { return x.first == s.first; });
                        if (sit == m.src.end()) m.src.push_back({s.first, 0.0 + s.second});
                        else sit->second = sit->second + s.second;
                    }
                }
            }
        }
        auto emit = [&](const Term& t) {
            for (const Op& o : t.ops) { B->pos.push_back(o.pos); B->tag.push_back(o.tag); }
            B->term_ptr.push_back((int32_t)B->pos.size());
            B->coeff.push_back(t.coeff);
            B->ferm.push_back(t.ferm ? 1 : 0);
            for (const auto& s : t.src) { B->src_idx.push_back(s.first); B->src_val.push_back(s.second); }
            B->src_ptr.push_back((int64_t)B->src_idx.size());
        };
        for (const Term& t : one_site) emit(t);
        for (auto& store : merged)
            for (const auto& kv : store) emit(kv.second);
        *out = B;
        return QCM_OK;
    } catch (const std::exception& e) {
        delete B;
        set_error(std::string("qcm_chem_terms: ") + e.what());
        return QCM_E_INVALID;
    }
}

int qcm_term_buf_view(const qcm_term_buf* B, qcm_term_view_t* v) {
    if (!B || !v) { set_error("qcm_term_buf_view: null argument"); return QCM_E_INVALID; }
    v->n_terms = (int64_t)B->coeff.size();
    v->term_ptr = B->term_ptr.data();
    v->pos = B->pos.data();
    v->tag = B->tag.data();
    v->coeff = B->coeff.data();
    v->fermionic = B->ferm.data();
    v->src_ptr = B->src_ptr.data();
    v->src_idx = B->src_idx.data();
    v->src_val = B->src_val.data();
    return QCM_OK;
}

void qcm_term_buf_destroy(qcm_term_buf* B) { delete B; }

}  // extern "C"
