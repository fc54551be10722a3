// Single-site MPO tensors from a list of model terms, in native code
// (TaggedMPOMaker, dmrg/framework/dmrg/models/generate_mpo/
// tagged_mpo_maker_optim.hpp: add_term :168-187, the two-operator and generic
// insertions :330-560, insert_filling :594-638, finalize :640-669, create_mpo
// :189-300, conjugate_key :671-735).
//
// A bond of the MPO is named by a key: the trivial left and right keys, or the
// operators (position, tag) already applied to the left of the bond, or still
// to be applied to its right.  Every term of two or more operators walks its
// sites, inserting at each site the (incoming key, outgoing key) element with
// the site's operator, and filling the sites between two operators with the
// identity or the fermionic filling on the open key.  Terms that share a key
// share the bond.  At the end the keys of each site are numbered in key order
// (the trivial left key 0, the trivial right key 1, then the rest), and each
// bond gets its spin and its Hermitian-conjugate partner with the phases of
// the SU(2) conjugation.
//
// One-site terms (site operators summed per site, and the core energy) need
// the operator algebra of the caller's model and are added by the caller as
// ready (TL, TR) element lists (qcm_mpo_maker_site_terms).
#include <algorithm>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "plan.hpp"

using qcm::set_error;

namespace {

// A key is the vector (kind, p0, t0, p1, t1, ...): ordered lexicographically,
// this is the order of the reference's (kind, [(pos, tag)...], offset) tuples.
using Key = std::vector<int32_t>;
constexpr int32_t KIND_TL = 0, KIND_BULK = 1, KIND_TR = 3;
constexpr int32_t KEY_TL = 0, KEY_TR = 1;  // interned first

struct KeyHash {
    size_t operator()(const Key& k) const noexcept {
        uint64_t h = 1469598103934665603ull;
        for (int32_t x : k) { h ^= (uint32_t)x; h *= 1099511628211ull; }
        return (size_t)h;
    }
};

struct Val { int32_t tag; double scale; int32_t label; };

struct TagTable {
    int32_t n = 0;
    std::vector<int32_t> ferm, twoS, action, herm, pdiff;
    int32_t ident = -1, ident_full = -1, fill = -1, symmetry = QCM_SYM_SU2U1;
};

struct SiteOut {
    int32_t row_dim = 0, col_dim = 0;
    std::vector<int32_t> elem_b1, elem_b2, elem_ptr, term_tag, term_label;
    std::vector<double> term_scale;
    std::vector<int32_t> right_spin, right_herm, right_phase;
};

TagTable read_tags(const qcm_tag_table_t* t) {
    if (!t || t->n_tags <= 0 || !t->fermionic || !t->spin || !t->herm_conj || !t->pdiff)
        throw std::runtime_error("malformed tag table");
    TagTable r;
    r.n = t->n_tags;
    r.ferm.assign(t->fermionic, t->fermionic + r.n);
    r.herm.assign(t->herm_conj, t->herm_conj + r.n);
    r.pdiff.assign(t->pdiff, t->pdiff + r.n);
    r.twoS.resize(r.n);
    r.action.resize(r.n);
    for (int32_t i = 0; i < r.n; ++i) {
        r.twoS[i] = t->spin[2 * i];
        r.action[i] = t->spin[2 * i + 1];
        if (r.herm[i] < 0 || r.herm[i] >= r.n) throw std::runtime_error("Hermitian conjugate tag out of range");
    }
    r.ident = t->identity;
    r.ident_full = t->identity_full;
    r.fill = t->fill;
    r.symmetry = t->symmetry;
    for (int32_t x : {r.ident, r.ident_full, r.fill})
        if (x < 0 || x >= r.n) throw std::runtime_error("identity / filling tag out of range");
    if (r.symmetry != QCM_SYM_SU2U1 && r.symmetry != QCM_SYM_TWOU1 && r.symmetry != QCM_SYM_U1)
        throw std::runtime_error("unknown symmetry");
    return r;
}

}  // namespace

struct qcm_mpo_maker {
    int32_t L = 0;
    TagTable tags;
    std::vector<Key> keys;
    std::unordered_map<Key, int32_t, KeyHash> key_id;
    // per site: (incoming key << 32 | outgoing key) -> element list in insertion order
    std::vector<std::unordered_map<uint64_t, std::vector<Val>>> prempo;
    bool built = false;
    bool finishing = false;   // finish was called: the element lists hold the chain-end identities
    std::vector<SiteOut> out;

    int32_t intern(const Key& k) {
        auto it = key_id.find(k);
        if (it != key_id.end()) return it->second;
        const int32_t id = (int32_t)keys.size();
        keys.push_back(k);
        key_id.emplace(k, id);
        return id;
    }

    static uint64_t pair_key(int32_t k1, int32_t k2) { return ((uint64_t)(uint32_t)k1 << 32) | (uint32_t)k2; }

    int32_t insert(int32_t p, int32_t k1, int32_t k2, Val v, bool attach) {
        auto& d = prempo[p];
        auto it = d.find(pair_key(k1, k2));
        if (it == d.end()) d.emplace(pair_key(k1, k2), std::vector<Val>{v});
        else if (!attach) it->second.push_back(v);
        return k2;
    }

    void insert_filling(int32_t i, int32_t j, int32_t k, bool trivial, bool spin_gt_one) {
        const int32_t op = trivial ? (spin_gt_one ? tags.ident_full : tags.ident) : tags.fill;
        for (int32_t s = i; s < j; ++s) {
            auto& d = prempo[s];
            auto it = d.find(pair_key(k, k));
            if (it == d.end()) d.emplace(pair_key(k, k), std::vector<Val>{{op, 1.0, -1}});
            else if (it->second[0].tag != op || it->second[0].scale != 1.0)
                throw std::runtime_error("pre-existing term at site " + std::to_string(s));
        }
    }

    int32_t bulk(const std::vector<std::pair<int32_t, int32_t>>& ops, size_t b, size_t e) {
        Key k;
        k.reserve(1 + 2 * (e - b));
        k.push_back(KIND_BULK);
        for (size_t i = b; i < e; ++i) { k.push_back(ops[i].first); k.push_back(ops[i].second); }
        return intern(k);
    }

    // one term of >= 2 operators, sorted by position (stable)
    void add_term(std::vector<std::pair<int32_t, int32_t>>& ops, double coeff, int32_t label) {
        const size_t n = ops.size();
        for (auto& o : ops) {
            if (o.first < 0 || o.first >= L) throw std::runtime_error("term position out of range");
            if (o.second < 0 || o.second >= tags.n) throw std::runtime_error("term tag out of range");
        }
        int32_t nferm = 0;
        for (auto& o : ops) nferm += tags.ferm[o.second] ? 1 : 0;
        int32_t spin = 0;
        if (n == 2) {
            spin += tags.action[ops[0].second];
            const int32_t k2 = bulk(ops, 1, 2);
            const int32_t k1 = insert(ops[0].first, KEY_TL, k2, {ops[0].second, coeff, label}, false);
            if (tags.ferm[ops[0].second]) --nferm;
            insert_filling(ops[0].first + 1, ops[1].first, k1, nferm % 2 == 0, spin > 1);
            spin += tags.action[ops[1].second];
            insert(ops[1].first, k1, KEY_TR, {ops[1].second, 1.0, -1}, true);
        } else {
            const size_t thresh = n / 2;
            int32_t k1 = KEY_TL;
            for (size_t i = 0; i < thresh; ++i) {
                spin += tags.action[ops[i].second];
                const int32_t k2 = bulk(ops, 0, i + 1);
                k1 = insert(ops[i].first, k1, k2, {ops[i].second, 1.0, -1}, true);
                if (tags.ferm[ops[i].second]) --nferm;
                insert_filling(ops[i].first + 1, ops[i + 1].first, k1, nferm % 2 == 0, spin > 1);
            }
            {
                const int32_t k2 = bulk(ops, thresh + 1, n);
                spin += tags.action[ops[thresh].second];
                k1 = insert(ops[thresh].first, k1, k2, {ops[thresh].second, coeff, label}, false);
                if (tags.ferm[ops[thresh].second]) --nferm;
                insert_filling(ops[thresh].first + 1, ops[thresh + 1].first, k1, nferm % 2 == 0, spin > 1);
            }
            for (size_t i = thresh + 1; i < n; ++i) {
                const int32_t k2 = (i == n - 1) ? KEY_TR : bulk(ops, i + 1, n);
                spin += tags.action[ops[i].second];
                k1 = insert(ops[i].first, k1, k2, {ops[i].second, 1.0, -1}, true);
                if (tags.ferm[ops[i].second]) --nferm;
                if (i != n - 1) insert_filling(ops[i].first + 1, ops[i + 1].first, k1, nferm % 2 == 0, spin > 1);
            }
        }
        if (spin != 0) throw std::runtime_error("term does not couple to total spin 0");
    }

    // Hermitian-conjugate key and the phases of the pair (the SU(2) conjugation
    // of one- and two-operator keys; abelian groups: phase 1)
    std::pair<Key, std::pair<int32_t, int32_t>> conjugate(const Key& k, int32_t p) const {
        Key c = k;
        for (size_t i = 2; i < c.size(); i += 2) c[i] = tags.herm[c[i]];
        int32_t ph0 = 1, ph1 = 1;
        const size_t nop = (k.size() - 1) / 2;
        if (tags.symmetry == QCM_SYM_SU2U1) {
            if (nop == 1) {
                const int32_t t = k[2];
                if (p < k[1]) {
                    if (tags.pdiff[t] == 1) { ph0 = 1; ph1 = -1; }
                    else if (tags.pdiff[t] == -1) { ph0 = -1; ph1 = 1; }
                } else if (tags.twoS[t] == 1) {
                    ph0 = -1; ph1 = 1;
                }
            }
            if (nop == 2) {
                const int32_t t1 = k[2], t2 = k[4];
                const int32_t d1 = tags.pdiff[t1], d2 = tags.pdiff[t2];
                if (tags.twoS[t1] == 1 && tags.twoS[t2] == 1 && tags.action[t2] == -1 && d1 == -d2) { ph0 = -1; ph1 = -1; }
                if (tags.twoS[t1] == 1 && tags.twoS[t2] == 1 && tags.action[t2] == 1 && d1 == d2) { ph0 = -1; ph1 = -1; }
            }
        }
        return {c, {ph0, ph1}};
    }

    void create(int32_t leftmost_right, int32_t rightmost_left) {
        for (int32_t p = 0; p < rightmost_left && p < L; ++p)
            prempo[p][pair_key(KEY_TL, KEY_TL)].push_back({tags.ident, 1.0, -1});
        for (int32_t p = std::max(0, leftmost_right + 1); p < L; ++p)
            prempo[p][pair_key(KEY_TR, KEY_TR)].push_back({tags.ident, 1.0, -1});
        // rank of every key in key order
        std::vector<int32_t> order(keys.size()), rank(keys.size());
        for (size_t i = 0; i < keys.size(); ++i) order[i] = (int32_t)i;
        std::sort(order.begin(), order.end(), [&](int32_t a, int32_t b) { return keys[a] < keys[b]; });
        for (size_t i = 0; i < order.size(); ++i) rank[order[i]] = (int32_t)i;

        out.assign(L, SiteOut());
        std::unordered_map<int32_t, int32_t> left{{KEY_TL, 0}};
        std::vector<int32_t> left_twoS{0}, left_diff{0};
        for (int32_t p = 0; p < L; ++p) {
            SiteOut& so = out[p];
            std::vector<uint64_t> pk;
            pk.reserve(prempo[p].size());
            for (auto& kv : prempo[p]) pk.push_back(kv.first);
            std::sort(pk.begin(), pk.end(), [&](uint64_t a, uint64_t b) {
                const int32_t a1 = (int32_t)(a >> 32), a2 = (int32_t)(uint32_t)a;
                const int32_t b1 = (int32_t)(b >> 32), b2 = (int32_t)(uint32_t)b;
                if (rank[a2] != rank[b2]) return rank[a2] < rank[b2];
                return rank[a1] < rank[b1];
            });
            struct Pre { int32_t b1, b2; Val v; };
            std::vector<Pre> pre;
            std::unordered_map<int32_t, int32_t> right;
            std::vector<std::pair<int32_t, std::pair<int32_t, int32_t>>> herm;  // (k2, phases), k2 key order
            std::unordered_map<int32_t, Key> herm_conj_key;
            std::unordered_set<int32_t> seen_k2;
            int32_t r = 2;
            for (uint64_t kk : pk) {
                const int32_t k1 = (int32_t)(kk >> 32), k2 = (int32_t)(uint32_t)kk;
                for (const Val& v : prempo[p][kk]) {
                    auto lt = left.find(k1);
                    if (lt == left.end()) throw std::runtime_error("incoming key not found at site " + std::to_string(p));
                    auto rt = right.find(k2);
                    if (rt == right.end()) {
                        const int32_t idx = k2 == KEY_TL ? 0 : (k2 == KEY_TR ? 1 : r++);
                        rt = right.emplace(k2, idx).first;
                    }
                    pre.push_back({lt->second, p == L - 1 ? 0 : rt->second, v});
                }
                // the conjugate key and its phases depend only on the key and the site
                if (!seen_k2.insert(k2).second) continue;
                auto cj = conjugate(keys[k2], p);
                if (cj.first != keys[k2]) {
                    herm.push_back({k2, cj.second});
                    herm_conj_key[k2] = cj.first;
                }
            }
            if (pre.empty()) throw std::runtime_error("no element at site " + std::to_string(p));
            int32_t ldim = 0, rdim = 0;
            for (auto& e : pre) { ldim = std::max(ldim, e.b1 + 1); rdim = std::max(rdim, e.b2 + 1); }
            // bond spins: the incoming bond's spin coupled with the operator's action
            std::vector<int32_t> rs(rdim, 0), rd(rdim, 0);
            for (auto& e : pre) {
                if (e.b1 >= (int32_t)left_twoS.size()) throw std::runtime_error("incoming bond without spin");
                const int32_t ts = left_twoS[e.b1] + tags.action[e.v.tag];
                if (!(rs[e.b2] == 0 || rs[e.b2] == ts))
                    throw std::runtime_error("inconsistent bond spin at site " + std::to_string(p));
                rs[e.b2] = ts;
                rd[e.b2] = left_diff[e.b1];
            }
            std::vector<int32_t> rherm(rdim), rphase(rdim, 1);
            for (int32_t b = 0; b < rdim; ++b) rherm[b] = b;
            std::sort(herm.begin(), herm.end(), [&](const auto& a, const auto& b) { return rank[a.first] < rank[b.first]; });
            for (auto& h : herm) {
                auto ro = right.find(h.first);
                const int32_t romeo = ro == right.end() ? 0 : ro->second;
                int32_t julia = 0;
                auto cid = key_id.find(herm_conj_key[h.first]);
                if (cid != key_id.end()) {
                    auto jt = right.find(cid->second);
                    if (jt != right.end()) julia = jt->second;
                }
                if (romeo < julia) {
                    if (julia >= rdim) throw std::runtime_error("Hermitian partner beyond the bond dimension");
                    std::swap(rherm[romeo], rherm[julia]);
                    rphase[romeo] = h.second.first;
                    rphase[julia] = h.second.second;
                }
            }
            // column-major elements; an element's terms latest first
            std::vector<int32_t> idx(pre.size());
            for (size_t i = 0; i < pre.size(); ++i) idx[i] = (int32_t)i;
            std::stable_sort(idx.begin(), idx.end(), [&](int32_t a, int32_t b) {
                if (pre[a].b2 != pre[b].b2) return pre[a].b2 < pre[b].b2;
                return pre[a].b1 < pre[b].b1;
            });
            so.row_dim = p == 0 ? 1 : ldim;
            so.col_dim = p == L - 1 ? 1 : rdim;
            for (size_t i = 0; i < idx.size();) {
                size_t j = i;
                while (j < idx.size() && pre[idx[j]].b1 == pre[idx[i]].b1 && pre[idx[j]].b2 == pre[idx[i]].b2) ++j;
                so.elem_b1.push_back(pre[idx[i]].b1);
                so.elem_b2.push_back(pre[idx[i]].b2);
                so.elem_ptr.push_back((int32_t)so.term_tag.size());
                for (size_t q = j; q-- > i;) {
                    const Val& v = pre[idx[q]].v;
                    so.term_tag.push_back(v.tag);
                    so.term_scale.push_back(v.scale);
                    so.term_label.push_back(v.label);
                }
                i = j;
            }
            so.elem_ptr.push_back((int32_t)so.term_tag.size());
            so.right_spin.resize(2 * (size_t)rdim);
            for (int32_t b = 0; b < rdim; ++b) { so.right_spin[2 * b] = rs[b]; so.right_spin[2 * b + 1] = rd[b]; }
            so.right_herm = rherm;
            so.right_phase = rphase;
            left = right;
            left_twoS = rs;
            left_diff = rd;
        }
        built = true;
    }
};

extern "C" {

int qcm_mpo_maker_create(int32_t L, const qcm_tag_table_t* tags, qcm_mpo_maker** out) {
    if (!out) { set_error("qcm_mpo_maker_create: null output"); return QCM_E_INVALID; }
    *out = nullptr;
    if (L <= 0) { set_error("qcm_mpo_maker_create: L must be positive"); return QCM_E_INVALID; }
    auto* M = new qcm_mpo_maker();
    try {
        M->L = L;
        M->tags = read_tags(tags);
        M->intern(Key{KIND_TL});
        M->intern(Key{KIND_TR});
        M->prempo.resize(L);
        *out = M;
        return QCM_OK;
    } catch (const std::exception& e) {
        delete M;
        set_error(std::string("qcm_mpo_maker_create: ") + e.what());
        return QCM_E_INVALID;
    }
}

int qcm_mpo_maker_add_terms(qcm_mpo_maker* M, int32_t n_terms, const int32_t* term_ptr, const int32_t* pos,
                            const int32_t* tag, const double* coeff, const int32_t* label) {
    if (!M || n_terms < 0 || (n_terms > 0 && (!term_ptr || !pos || !tag || !coeff || !label))) {
        set_error("qcm_mpo_maker_add_terms: null argument");
        return QCM_E_INVALID;
    }
    if (M->built || M->finishing) { set_error("qcm_mpo_maker_add_terms: maker already finished"); return QCM_E_STATE; }
    try {
        if (n_terms > 0 && term_ptr[0] != 0) throw std::runtime_error("term_ptr[0] != 0");
        std::vector<std::pair<int32_t, int32_t>> ops;
        for (int32_t t = 0; t < n_terms; ++t) {
            const int32_t b = term_ptr[t], e = term_ptr[t + 1];
            if (e - b < 2) throw std::runtime_error("terms of fewer than two operators are site terms");
            ops.clear();
            for (int32_t i = b; i < e; ++i) ops.push_back({pos[i], tag[i]});
            std::stable_sort(ops.begin(), ops.end(), [](const auto& a, const auto& c) { return a.first < c.first; });
            M->add_term(ops, coeff[t], label[t]);
        }
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string("qcm_mpo_maker_add_terms: ") + e.what());
        return QCM_E_INVALID;
    }
}

int qcm_mpo_maker_site_terms(qcm_mpo_maker* M, int32_t site, int32_t n, const int32_t* tag, const double* scale,
                             const int32_t* label) {
    if (!M || n <= 0 || !tag || !scale || !label) { set_error("qcm_mpo_maker_site_terms: null argument"); return QCM_E_INVALID; }
    if (M->built || M->finishing) { set_error("qcm_mpo_maker_site_terms: maker already finished"); return QCM_E_STATE; }
    if (site < 0 || site >= M->L) { set_error("qcm_mpo_maker_site_terms: site out of range"); return QCM_E_INVALID; }
    auto& d = M->prempo[site];
    const uint64_t kk = qcm_mpo_maker::pair_key(KEY_TL, KEY_TR);
    if (d.count(kk)) { set_error("qcm_mpo_maker_site_terms: another site term already exists"); return QCM_E_INVALID; }
    std::vector<Val> v;
    for (int32_t i = 0; i < n; ++i) v.push_back({tag[i], scale[i], label[i]});
    d.emplace(kk, std::move(v));
    return QCM_OK;
}

int qcm_mpo_maker_finish(qcm_mpo_maker* M, const qcm_tag_table_t* tags, int32_t leftmost_right, int32_t rightmost_left) {
    if (!M) { set_error("qcm_mpo_maker_finish: null handle"); return QCM_E_INVALID; }
    if (M->built || M->finishing) {
        set_error("qcm_mpo_maker_finish: called before on this maker (after a failed finish, destroy it)");
        return QCM_E_STATE;
    }
    M->finishing = true;
    try {
        if (tags) {
            TagTable t = read_tags(tags);
            if (t.n < M->tags.n) throw std::runtime_error("tag table shrank");
            M->tags = std::move(t);
        }
        for (auto& d : M->prempo)
            for (auto& kv : d)
                for (const Val& v : kv.second)
                    if (v.tag < 0 || v.tag >= M->tags.n) throw std::runtime_error("site term tag out of range");
        M->create(leftmost_right, rightmost_left);
        return QCM_OK;
    } catch (const std::exception& e) {
        M->out.clear();
        set_error(std::string("qcm_mpo_maker_finish: ") + e.what());
        return QCM_E_INVALID;
    }
}

int qcm_mpo_maker_site(const qcm_mpo_maker* M, int32_t site, qcm_mpo_site_t* view) {
    if (!M || !view) { set_error("qcm_mpo_maker_site: null argument"); return QCM_E_INVALID; }
    if (!M->built) { set_error("qcm_mpo_maker_site: tensors not built (qcm_mpo_maker_finish)"); return QCM_E_STATE; }
    if (site < 0 || site >= M->L) { set_error("qcm_mpo_maker_site: site out of range"); return QCM_E_INVALID; }
    const SiteOut& s = M->out[site];
    view->row_dim = s.row_dim;
    view->col_dim = s.col_dim;
    view->bond_dim = (int32_t)s.right_herm.size();
    view->n_elem = (int32_t)s.elem_b1.size();
    view->elem_b1 = s.elem_b1.data();
    view->elem_b2 = s.elem_b2.data();
    view->elem_ptr = s.elem_ptr.data();
    view->term_tag = s.term_tag.data();
    view->term_scale = s.term_scale.data();
    view->term_label = s.term_label.data();
    view->right_spin = s.right_spin.data();
    view->right_herm = s.right_herm.data();
    view->right_phase = s.right_phase.data();
    return QCM_OK;
}

void qcm_mpo_maker_destroy(qcm_mpo_maker* M) { delete M; }

}  // extern "C"
