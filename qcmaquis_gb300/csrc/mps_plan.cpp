// Plans of the MPS-level steps around the eigensolver: forming the two-site
// tensor, undoing its SU(2) reduction before the truncation, and assembling the
// two new site tensors after it.  For the abelian TwoU1 group the two-site
// tensor is not reduced: its physical index is the plain product of the two
// sites' and only the reshapes remain (twositetensor.hpp:125-130, 352-366).  Every step is a fixed linear map between two
// block layouts (plus, for the two-site tensor, one grouped block product), so
// it is planned once on the host as gather tiles -- each output tile the sum of
// scaled source tiles, its couplings precomputed -- and runs as one gather
// launch per map on the device, with no per-block work on the host.
//
// Reference steps (paths below dmrg/framework/dmrg/mp_tensors/):
//   TwoSiteTensor(mps1, mps2) + make_mps       twositetensor.hpp:22-31, 132-139
//     theta = A(left-paired) . B(right-paired)  (block_matrix_algorithms.h:47-80)
//     reshape_both_to_right                      ts_reshape.h:231-290
//     SU(2) reduce_right (6j recoupling)         ts_reduction.h:42-141
//     reshape_right_to_left                      reshapes.h:290-338
//   operator<< + split_mps_l2r/r2l prologue    twositetensor.hpp:141-180, 372-389
//     SU(2) unreduce_left                        ts_reduction.h:143-251
//     reshape_left_to_both                       ts_reshape.h:89-145
//   split_mps_l2r/r2l epilogue                 twositetensor.hpp:141-180
//     A = U, B = S V (l2r) or A = U S, B = V (r2l), B reshaped right -> left
//   mergeUnitaryFactor                         SweepBasedAlgorithms/SweepMPSUpdater.h:237-250
//     multiply_from_left: N . T_rp, reshaped back  mpstensor.hpp:314-321
//     multiply_from_right: T_lp . N                mpstensor.hpp:302-309
//     the reshapes of right normalisation          mpstensor.hpp:239-258
//
// Every output block of a map is cleared first (a ZERO stage), so elements that
// no tile writes read as zero, as the reference's freshly allocated blocks do.
#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "plan.hpp"

namespace qcm {

namespace {

// Gather tiles of one map, grouped by destination (several sources may add into
// one destination tile, e.g. the two 6j couplings of one reduced state).
struct TileMap {
    struct Dst { int64_t off, ldd, rows, cols; };
    std::map<int64_t, size_t> by_off;
    std::vector<Dst> dst;
    std::vector<std::vector<AxpyTerm>> terms;
    void add(int64_t doff, int64_t ldd, int64_t rows, int64_t cols, int32_t sbuf, int64_t soff, int64_t lds,
             double a) {
        if (rows <= 0 || cols <= 0) return;
        auto it = by_off.find(doff);
        size_t k;
        if (it == by_off.end()) {
            k = dst.size();
            by_off.emplace(doff, k);
            dst.push_back({doff, ldd, rows, cols});
            terms.emplace_back();
        } else {
            k = it->second;
            const Dst& d = dst[k];
            if (d.ldd != ldd || d.rows != rows || d.cols != cols)
                throw std::runtime_error("map tiles of different shapes share a destination");
        }
        terms[k].push_back({sbuf, soff, lds, a});
    }
    // an AXPY stage writing into dbuf, in destination order
    Stage stage(int32_t dbuf, qcm_plan* P) const {
        Stage st;
        st.kind = ST_AXPY;
        for (size_t k = 0; k < dst.size(); ++k) {
            AxpyOut o;
            o.dst_buf = dbuf;
            o.dst_off = dst[k].off;
            o.ldd = dst[k].ldd;
            o.rows = dst[k].rows;
            o.cols = dst[k].cols;
            o.t_begin = (int64_t)st.aterm.size();
            for (auto& t : terms[k]) st.aterm.push_back(t);
            o.t_end = (int64_t)st.aterm.size();
            st.aout.push_back(o);
            P->axpy_flops += 2.0 * o.rows * o.cols * (o.t_end - o.t_begin);
            P->axpy_bytes += 8.0 * o.rows * o.cols * (1 + (o.t_end - o.t_begin));
        }
        return st;
    }
};

Stage zero_stage(int32_t buf, int64_t len) {
    Stage z;
    z.kind = ST_ZERO;
    z.zbuf = buf;
    z.zoff = 0;
    z.zlen = len;
    return z;
}

// A pending output block: created on first use, offsets assigned once all exist.
struct Pending {
    BM bm;
    Blk& get(Q lc, Q rc, int64_t rows, int64_t cols) {
        size_t p = bm.find(lc, rc);
        if (p == bm.b.size()) {
            Blk nb;
            nb.lc = lc;
            nb.rc = rc;
            nb.rows = rows;
            nb.cols = cols;
            p = bm.insert(nb);
        }
        Blk& b = bm.b[p];
        if (b.rows != rows || b.cols != cols) throw std::runtime_error("inconsistent output block shape");
        return b;
    }
};

// A recorded piece: destination block key, position inside it, source element offset.
struct Piece {
    Q lc, rc;
    int64_t r0, c0, rows, cols;
    int32_t sbuf;
    int64_t soff, lds;
    double a;
};

void emit(const std::vector<Piece>& ps, const BM& out, TileMap& tm) {
    for (auto& p : ps) {
        const Blk& d = out.b[out.find(p.lc, p.rc)];
        tm.add(d.off + p.r0 + p.c0 * d.rows, d.rows, p.rows, p.cols, p.sbuf, p.soff, p.lds, p.a);
    }
}

inline int spin_of(Q c) { return c.s; }

double sign6(int jl, int jr, int S1, int S2) { return (((jl + jr + S1 + S2) / 2) % 2) ? -1.0 : 1.0; }

// reshape_left_to_right: left-paired (phys x left, right) -> right-paired (left, phys x right)
BM map_l2r(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& in, int32_t sbuf,
           std::vector<Piece>& ps) {
    PB in_left(phys, left_i, false), out_right(phys, right_i, true);
    Pending out;
    for (auto& blk : in.b) {
        size_t r = right_i.position(blk.rc);
        if (r == right_i.size()) continue;
        Q in_r = right_i.d[r].first;
        for (auto& pe : phys.d) {
            size_t l = left_i.position(fuse(blk.lc, neg(pe.first)));
            if (l == left_i.size()) continue;
            Q ol = left_i.d[l].first, orr = fuse(neg(pe.first), in_r);
            int64_t ld = left_i.d[l].second, rd = right_i.d[r].second;
            out.get(ol, orr, ld, out_right.size(orr));
            int64_t ilo = in_left(pe.first, ol), oro = out_right(pe.first, in_r);
            for (int64_t ss = 0; ss < pe.second; ++ss)
                ps.push_back({ol, orr, 0, oro + ss * rd, ld, rd, sbuf, blk.off + ilo + ss * ld, blk.rows, 1.0});
        }
    }
    return out.bm;
}

// reshape_right_to_left: right-paired (left, phys x right) -> left-paired (phys x left, right)
BM map_r2l(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& in, int32_t sbuf,
           std::vector<Piece>& ps) {
    PB in_right(phys, right_i, true), out_left(phys, left_i, false);
    Pending out;
    for (auto& blk : in.b) {
        size_t l = left_i.position(blk.lc);
        if (l == left_i.size()) continue;
        Q in_l = left_i.d[l].first;
        for (auto& pe : phys.d) {
            size_t r = right_i.position(fuse(blk.rc, pe.first));
            if (r == right_i.size()) continue;
            Q ol = fuse(pe.first, in_l), orr = right_i.d[r].first;
            int64_t ld = left_i.d[l].second, rd = right_i.d[r].second;
            out.get(ol, orr, out_left.size(ol), rd);
            int64_t iro = in_right(pe.first, orr), olo = out_left(pe.first, in_l);
            for (int64_t ss = 0; ss < pe.second; ++ss)
                ps.push_back({ol, orr, olo + ss * ld, 0, ld, rd, sbuf, blk.off + (iro + ss * rd) * blk.rows,
                              blk.rows, 1.0});
        }
    }
    return out.bm;
}

// reshape_both_to_right: (phys1 x left, phys2 x right) -> (left, phys1 phys2 x right)
BM map_both_to_right(const Idx& p1, const Idx& p2, const Idx& left_i, const Idx& right_i, const BM& in,
                     int32_t sbuf, std::vector<Piece>& ps) {
    Idx phys2 = index_product(p1, p2);
    PB phys_pb(p1, p2, false), in_left(p1, left_i, false), in_right(p2, right_i, true),
        out_right(phys2, right_i, true);
    Pending out;
    for (auto& blk : in.b) {
        for (auto& c1 : p1.d) {
            size_t l = left_i.position(fuse(blk.lc, neg(c1.first)));
            if (l == left_i.size()) continue;
            for (auto& c2 : p2.d) {
                size_t r = right_i.position(fuse(blk.rc, c2.first));
                if (r == right_i.size()) continue;
                Q sc = fuse(c1.first, c2.first);
                Q ol = left_i.d[l].first, orr = fuse(neg(sc), right_i.d[r].first);
                int64_t ld = left_i.d[l].second, rd = right_i.d[r].second;
                out.get(ol, orr, ld, out_right.size(orr));
                int64_t ilo = in_left(c1.first, left_i.d[l].first), iro = in_right(c2.first, right_i.d[r].first);
                int64_t oro = out_right(sc, right_i.d[r].first), opo = phys_pb(c1.first, c2.first);
                for (int64_t s1 = 0; s1 < c1.second; ++s1)
                    for (int64_t s2 = 0; s2 < c2.second; ++s2) {
                        int64_t so = opo + s1 * c2.second + s2;
                        ps.push_back({ol, orr, 0, oro + so * rd, ld, rd, sbuf,
                                      blk.off + ilo + s1 * ld + (iro + s2 * rd) * blk.rows, blk.rows, 1.0});
                    }
            }
        }
    }
    return out.bm;
}

// reshape_left_to_both: (phys1 phys2 x left, right) -> (phys1 x left, phys2 x right)
BM map_left_to_both(const Idx& p1, const Idx& p2, const Idx& left_i, const Idx& right_i, const BM& in,
                    int32_t sbuf, std::vector<Piece>& ps) {
    Idx phys2 = index_product(p1, p2);
    PB phys_pb(p1, p2, false), in_left(phys2, left_i, false), out_right(p2, right_i, true),
        out_left(p1, left_i, false);
    Pending out;
    for (auto& blk : in.b) {
        size_t r = right_i.position(blk.rc);
        if (r == right_i.size()) throw std::runtime_error("two-site tensor inconsistent with its right index");
        for (auto& c1 : p1.d)
            for (auto& c2 : p2.d) {
                Q sc = fuse(c1.first, c2.first);
                size_t l = left_i.position(fuse(blk.lc, neg(sc)));
                if (l == left_i.size()) continue;
                Q ol = fuse(c1.first, left_i.d[l].first), orr = fuse(neg(c2.first), right_i.d[r].first);
                int64_t ld = left_i.d[l].second, rd = right_i.d[r].second;
                out.get(ol, orr, out_left.size(ol), out_right.size(orr));
                int64_t ilo = in_left(sc, left_i.d[l].first), ipo = phys_pb(c1.first, c2.first);
                int64_t olo = out_left(c1.first, left_i.d[l].first), oro = out_right(c2.first, right_i.d[r].first);
                for (int64_t s1 = 0; s1 < c1.second; ++s1)
                    for (int64_t s2 = 0; s2 < c2.second; ++s2) {
                        int64_t si = ipo + s1 * c2.second + s2;
                        ps.push_back({ol, orr, olo + s1 * ld, oro + s2 * rd, ld, rd, sbuf, blk.off + ilo + si * ld,
                                      blk.rows, 1.0});
                    }
            }
    }
    return out.bm;
}

// SU(2) reduce_right on a right-paired two-site tensor (same layout in and out):
// column stripes of the product states recoupled by 6j symbols.
BM map_reduce_right(const Idx& p1, const Idx& p2, const Idx& right_i, const BM& in, int32_t sbuf,
                    std::vector<Piece>& ps) {
    Idx phys2 = index_product(p1, p2);
    PB phys_pb(p1, p2, false), in_right(phys2, right_i, true);
    BM out = in;
    for (auto& blk : in.b) {
        Q lc = blk.lc, in_r = blk.rc;
        for (auto& sc : phys2.d) {
            size_t r = right_i.position(fuse(in_r, sc.first));
            if (r == right_i.size()) continue;
            int64_t iro = in_right(sc.first, right_i.d[r].first), rs = right_i.d[r].second;
            for (auto& c1 : p1.d)
                for (auto& c2 : p2.d) {
                    if (sc.first != fuse(c1.first, c2.first)) continue;
                    int64_t ipo = phys_pb(c1.first, c2.first);
                    int S1 = std::abs(spin_of(c1.first)), S2 = std::abs(spin_of(c2.first));
                    int jl = spin_of(lc), jm = spin_of(lc) + spin_of(c1.first), jr = spin_of(right_i.d[r].first);
                    if (jm < 0) continue;
                    std::vector<std::pair<int64_t, int>> outs;
                    if (jl == jr && jl > 0 && S1 == 1 && S2 == 1) {
                        int64_t base = spin_of(c1.first) == 1 ? ipo : ipo - 1;
                        for (int j = std::abs(S1 - S2); j <= S1 + S2; j += 2) outs.push_back({base + j / 2, j});
                    } else {
                        outs.push_back({ipo, std::abs(spin_of(c1.first) + spin_of(c2.first))});
                    }
                    for (auto& oj : outs) {
                        const int j = oj.second;
                        double cc = std::sqrt((j + 1.0) * (jm + 1.0)) * wigner6j(jl, jr, j, S2, S1, jm) *
                                    sign6(jl, jr, S1, S2);
                        if (cc == 0.0) continue;
                        for (int64_t s1 = 0; s1 < c1.second; ++s1)
                            for (int64_t s2 = 0; s2 < c2.second; ++s2) {
                                int64_t si = ipo + s1 * c2.second + s2, so = oj.first + s1 * c2.second + s2;
                                ps.push_back({lc, in_r, 0, iro + so * rs, blk.rows, rs, sbuf,
                                              blk.off + (iro + si * rs) * blk.rows, blk.rows, cc});
                            }
                    }
                }
        }
    }
    return out;
}

// SU(2) unreduce_left on a left-paired reduced two-site tensor (same layout in
// and out): row stripes recoupled by 6j symbols.
BM map_unreduce_left(const Idx& p1, const Idx& p2, const Idx& left_i, const BM& in, int32_t sbuf,
                     std::vector<Piece>& ps) {
    Idx phys2 = index_product(p1, p2);
    PB phys_pb(p1, p2, false), in_left(phys2, left_i, false);
    BM out = in;
    for (auto& blk : in.b) {
        Q in_l = blk.lc, rc = blk.rc;
        for (auto& sc : phys2.d) {
            size_t l = left_i.position(fuse(in_l, neg(sc.first)));
            if (l == left_i.size()) continue;
            int64_t ilo = in_left(sc.first, left_i.d[l].first), ld = left_i.d[l].second;
            for (auto& c1 : p1.d)
                for (auto& c2 : p2.d) {
                    if (sc.first != fuse(c1.first, c2.first)) continue;
                    int64_t ipo = phys_pb(c1.first, c2.first);
                    int S1 = std::abs(spin_of(c1.first)), S2 = std::abs(spin_of(c2.first));
                    int jl = spin_of(left_i.d[l].first), jr = spin_of(rc);
                    struct O { int64_t opo; int j, jm; };
                    std::vector<O> outs;
                    if (jl == jr && jl > 0 && S1 == 1 && S2 == 1) {
                        int j = spin_of(c1.first) == 1 ? 0 : 2;
                        int64_t base = j == 0 ? ipo : ipo - 1;
                        for (int jm : {jl - 1, jl + 1}) outs.push_back({jm == jl - 1 ? base + 1 : base, j, jm});
                    } else {
                        int j = std::abs(spin_of(c1.first) + spin_of(c2.first));
                        int jm = jl + spin_of(c1.first);
                        if (jm < 0) continue;
                        outs.push_back({ipo, j, jm});
                    }
                    for (auto& o : outs) {
                        double cc = std::sqrt((o.j + 1.0) * (o.jm + 1.0)) * wigner6j(jl, jr, o.j, S2, S1, o.jm) *
                                    sign6(jl, jr, S1, S2);
                        if (cc == 0.0) continue;
                        for (int64_t s1 = 0; s1 < c1.second; ++s1)
                            for (int64_t s2 = 0; s2 < c2.second; ++s2) {
                                int64_t si = ipo + s1 * c2.second + s2, so = o.opo + s1 * c2.second + s2;
                                ps.push_back({in_l, rc, ilo + so * ld, 0, ld, blk.cols, sbuf,
                                              blk.off + ilo + si * ld, blk.rows, cc});
                            }
                    }
                }
        }
    }
    return out;
}

Idx left_basis(const BM& m) {
    Idx r;
    for (auto& b : m.b) r.d.push_back({b.lc, b.rows});
    return r;
}
Idx right_basis(const BM& m) {
    Idx r;
    for (auto& b : m.b) r.d.push_back({b.rc, b.cols});
    return r;
}

// one map: clear the destination, then the gather tiles
void add_map(qcm_plan* P, const std::vector<Piece>& ps, BM& out, int32_t dbuf, int64_t& len) {
    len = out.assign_offsets(0);
    P->stages.push_back(zero_stage(dbuf, len));
    TileMap tm;
    emit(ps, out, tm);
    if (!tm.dst.empty()) P->stages.push_back(tm.stage(dbuf, P));
}

// C = A . B, block by block where A's right charge is B's left charge (the charge
// matching of block_matrix_algorithms.h:47-80): C's blocks into cbuf (cleared first),
// one grouped-product output per C block summing its segments in the order found.
void add_product(qcm_plan* P, const BM& A, int32_t abuf, const BM& B, int32_t bbuf, int32_t cbuf, BM& C,
                 int64_t& len) {
    struct Job { size_t a, b; };
    std::vector<Job> jobs;
    for (size_t ka = 0; ka < A.b.size(); ++ka) {
        const Blk& a = A.b[ka];
        for (size_t kb = B.left_lower_bound(a.rc); kb < B.b.size() && B.b[kb].lc == a.rc; ++kb) {
            const Blk& b = B.b[kb];
            if (a.cols != b.rows) throw std::runtime_error("block product: inner dimensions differ");
            if (C.find(a.lc, b.rc) == C.b.size()) {
                Blk nb;
                nb.lc = a.lc;
                nb.rc = b.rc;
                nb.rows = a.rows;
                nb.cols = b.cols;
                C.insert(nb);
            }
            jobs.push_back({ka, kb});
        }
    }
    len = C.assign_offsets(0);
    P->stages.push_back(zero_stage(cbuf, len));
    Stage g;
    g.kind = ST_GEMM;
    std::vector<std::vector<GemmSeg>> segs(C.b.size());
    for (auto& j : jobs) {
        const Blk& a = A.b[j.a];
        const Blk& b = B.b[j.b];
        GemmSeg s;
        s.a_buf = abuf;
        s.ta = 0;
        s.a_off = a.off;
        s.lda = a.rows;
        s.b_buf = bbuf;
        s.tb = 0;
        s.b_off = b.off;
        s.ldb = b.rows;
        s.K = a.cols;
        s.alpha = 1.0;
        segs[C.find(a.lc, b.rc)].push_back(s);
        P->gemm_flops += 2.0 * a.rows * b.cols * a.cols;
    }
    for (size_t c = 0; c < C.b.size(); ++c) {
        if (segs[c].empty()) continue;
        GemmOut o;
        o.c_buf = cbuf;
        o.c_off = C.b[c].off;
        o.ldc = C.b[c].rows;
        o.M = C.b[c].rows;
        o.N = C.b[c].cols;
        o.s_begin = (int64_t)g.gseg.size();
        for (auto& s : segs[c]) g.gseg.push_back(s);
        o.s_end = (int64_t)g.gseg.size();
        g.gout.push_back(o);
    }
    if (!g.gout.empty()) P->stages.push_back(std::move(g));
}

}  // namespace

// theta of sites (i, i+1) as the reduced two-site tensor, left-paired.
// Slots: KET = A (left-paired), LEFT = B (left-paired), OUT = the two-site tensor.
qcm_plan* build_theta(const Idx& p1, const Idx& a_left, const Idx& a_right, const BM& A, const Idx& p2,
                      const Idx& b_left, const Idx& b_right, const BM& B, bool abelian) {
    auto P = std::make_unique<qcm_plan>();
    P->kind = PK_THETA;
    int64_t s0 = 0, s1 = 0, s2 = 0, len = 0;
    // B right-paired -> S0
    std::vector<Piece> ps;
    BM b_rp = map_l2r(p2, b_left, b_right, B, QCM_BUF_LEFT, ps);
    add_map(P.get(), ps, b_rp, QCM_BUF_S0, len);
    s0 = std::max(s0, len);
    // theta(lc, rc) = sum_x A(lc, x) B_rp(x, rc) -> S1, one output per theta block
    BM th;
    struct Job { size_t a, b; };
    std::vector<Job> jobs;
    for (size_t ka = 0; ka < A.b.size(); ++ka) {
        const Blk& a = A.b[ka];
        for (size_t kb = b_rp.left_lower_bound(a.rc); kb < b_rp.b.size() && b_rp.b[kb].lc == a.rc; ++kb) {
            const Blk& b = b_rp.b[kb];
            if (a.cols != b.rows) throw std::runtime_error("theta: inner dimensions differ");
            size_t p = th.find(a.lc, b.rc);
            if (p == th.b.size()) {
                Blk nb;
                nb.lc = a.lc;
                nb.rc = b.rc;
                nb.rows = a.rows;
                nb.cols = b.cols;
                th.insert(nb);
            }
            jobs.push_back({ka, kb});
        }
    }
    s1 = th.assign_offsets(0);
    {
        Stage g;
        g.kind = ST_GEMM;
        // segments grouped per output block, in the order the products were found
        std::vector<std::vector<GemmSeg>> segs(th.b.size());
        for (auto& j : jobs) {
            const Blk& a = A.b[j.a];
            const Blk& b = b_rp.b[j.b];
            size_t c = th.find(a.lc, b.rc);
            GemmSeg s;
            s.a_buf = QCM_BUF_KET;
            s.ta = 0;
            s.a_off = a.off;
            s.lda = a.rows;
            s.b_buf = QCM_BUF_S0;
            s.tb = 0;
            s.b_off = b.off;
            s.ldb = b.rows;
            s.K = a.cols;
            s.alpha = 1.0;
            segs[c].push_back(s);
            P->gemm_flops += 2.0 * a.rows * b.cols * a.cols;
        }
        for (size_t c = 0; c < th.b.size(); ++c) {
            const Blk& cb = th.b[c];
            GemmOut o;
            o.c_buf = QCM_BUF_S1;
            o.c_off = cb.off;
            o.ldc = cb.rows;
            o.M = cb.rows;
            o.N = cb.cols;
            o.s_begin = (int64_t)g.gseg.size();
            for (auto& s : segs[c]) g.gseg.push_back(s);
            o.s_end = (int64_t)g.gseg.size();
            if (o.s_end == o.s_begin) continue;
            g.gout.push_back(o);
        }
        P->stages.push_back(zero_stage(QCM_BUF_S1, s1));
        P->stages.push_back(std::move(g));
    }
    // both -> right (S2), reduce_right (S0; SU(2) only), right -> left (OUT)
    ps.clear();
    BM rp = map_both_to_right(p1, p2, a_left, b_right, th, QCM_BUF_S1, ps);
    add_map(P.get(), ps, rp, QCM_BUF_S2, len);
    s2 = std::max(s2, len);
    BM red;
    int32_t red_buf = QCM_BUF_S2;
    if (abelian) {
        red = rp;
    } else {
        ps.clear();
        red = map_reduce_right(p1, p2, b_right, rp, QCM_BUF_S2, ps);
        add_map(P.get(), ps, red, QCM_BUF_S0, len);
        s0 = std::max(s0, len);
        red_buf = QCM_BUF_S0;
    }
    Idx phys2 = index_product(p1, p2);
    Idx new_left = left_basis(red);
    Idx right = b_right;
    Idx possible_right = index_product(phys2, new_left);
    common_subset(right, possible_right);
    ps.clear();
    BM lp = map_r2l(phys2, new_left, right, red, red_buf, ps);
    add_map(P.get(), ps, lp, QCM_BUF_OUT, len);
    P->out_elems = len;
    P->scratch[0] = s0;
    P->scratch[1] = s1;
    P->scratch[2] = s2;
    P->out_bm = lp.b;
    P->out_phys = phys2;
    P->out_left = new_left;
    P->out_right = right;
    return P.release();
}

// The both-paired two-site tensor (the matrix the truncation factorises) from the
// reduced left-paired one.  Slots: KET = the reduced tensor, OUT = theta (both-paired).
qcm_plan* build_split(const Idx& p1, const Idx& p2, const Idx& left_i, const Idx& right_i, const BM& u,
                      bool abelian) {
    auto P = std::make_unique<qcm_plan>();
    P->kind = PK_SPLIT;
    int64_t len = 0;
    std::vector<Piece> ps;
    BM tst = u;
    int32_t tst_buf = QCM_BUF_KET;
    if (!abelian) {
        tst = map_unreduce_left(p1, p2, left_i, u, QCM_BUF_KET, ps);
        add_map(P.get(), ps, tst, QCM_BUF_S0, len);
        P->scratch[0] = len;
        tst_buf = QCM_BUF_S0;
    }
    ps.clear();
    BM both = map_left_to_both(p1, p2, left_i, right_i, tst, tst_buf, ps);
    add_map(P.get(), ps, both, QCM_BUF_OUT, len);
    P->out_elems = len;
    P->out_bm = both.b;
    P->out_phys = p1;
    P->out_left = left_i;
    P->out_right = right_i;
    P->out2_phys = p2;
    return P.release();
}

// The two site tensors of a truncated SVD split.  Inputs (slots): KET = U, LEFT = Vt
// of the batched SVD of the both-paired blocks (u_off / vt_off, k[i] = min(rows,
// cols)), S values on the host; keep[i] singular triplets kept of block i.
// l2r: A = U[:, :keep] (left-paired, OUT), B = S V[:keep, :] right-paired, reshaped to
// left-paired into S2 (the second output).  r2l: A = U[:, :keep] S, B = V[:keep, :].
qcm_plan* build_assemble(const Idx& p1, const Idx& p2, const Idx& left_i, const Idx& right_i, const BM& both,
                         const int64_t* u_off, const int64_t* vt_off, const int64_t* kdim, const int64_t* keep,
                         const double* S_host, const int64_t* s_off, bool l2r) {
    auto P = std::make_unique<qcm_plan>();
    P->kind = PK_ASSEMBLE;
    BM a, brp;
    for (size_t i = 0; i < both.b.size(); ++i) {
        const Blk& x = both.b[i];
        if (keep[i] <= 0) continue;
        Blk ab;
        ab.lc = x.lc;
        ab.rc = x.rc;
        ab.rows = x.rows;
        ab.cols = keep[i];
        a.insert(ab);
        Blk bb;
        bb.lc = x.rc;
        bb.rc = x.rc;
        bb.rows = keep[i];
        bb.cols = x.cols;
        brp.insert(bb);
    }
    int64_t alen = a.assign_offsets(0), blen = brp.assign_offsets(0);
    TileMap ta, tb;
    for (size_t i = 0; i < both.b.size(); ++i) {
        const Blk& x = both.b[i];
        const int64_t kk = keep[i], k = kdim[i];
        if (kk <= 0) continue;
        const Blk& ad = a.b[a.find(x.lc, x.rc)];
        const Blk& bd = brp.b[brp.find(x.rc, x.rc)];
        if (l2r) {
            // A = U[:, :kk]: one contiguous column-major prefix
            ta.add(ad.off, ad.rows, ad.rows, kk, QCM_BUF_KET, u_off[i], x.rows, 1.0);
            // B = S V: row t of Vt scaled by s_t
            for (int64_t t = 0; t < kk; ++t)
                tb.add(bd.off + t, bd.rows, 1, bd.cols, QCM_BUF_LEFT, vt_off[i] + t, k, S_host[s_off[i] + t]);
        } else {
            for (int64_t t = 0; t < kk; ++t)
                ta.add(ad.off + t * ad.rows, ad.rows, ad.rows, 1, QCM_BUF_KET, u_off[i] + t * x.rows, x.rows,
                       S_host[s_off[i] + t]);
            tb.add(bd.off, bd.rows, kk, bd.cols, QCM_BUF_LEFT, vt_off[i], k, 1.0);
        }
    }
    P->stages.push_back(zero_stage(QCM_BUF_OUT, alen));
    if (!ta.dst.empty()) P->stages.push_back(ta.stage(QCM_BUF_OUT, P.get()));
    P->stages.push_back(zero_stage(QCM_BUF_S0, blen));
    if (!tb.dst.empty()) P->stages.push_back(tb.stage(QCM_BUF_S0, P.get()));
    // A: MPSTensor(p1, left, A.right_basis(), A, LeftPaired) with the left index reduced
    // to the charges the new bond reaches (common_subset with adjoin(p1) x right)
    Idx a_right = right_basis(a);
    Idx a_left = left_i;
    Idx reach = index_product(adjoin(p1), a_right);
    common_subset(a_left, reach);
    // B: MPSTensor(p2, Brp.left_basis(), right, Brp, RightPaired), then left-paired
    Idx b_left = left_basis(brp);
    Idx b_right = right_i;
    Idx reach_b = index_product(p2, b_left);
    common_subset(b_right, reach_b);
    std::vector<Piece> ps;
    BM blp = map_r2l(p2, b_left, b_right, brp, QCM_BUF_S0, ps);
    int64_t len = 0;
    add_map(P.get(), ps, blp, QCM_BUF_S2, len);
    P->out_elems = alen;
    P->scratch[0] = blen;
    P->scratch[2] = len;
    P->out_bm = a.b;
    P->out_phys = p1;
    P->out_left = a_left;
    P->out_right = a_right;
    P->out2_bm = blp.b;
    P->out2_phys = p2;
    P->out2_left = b_left;
    P->out2_right = b_right;
    return P.release();
}

// The product of a site tensor T (left-paired, slot KET) with a block-diagonal bond
// factor N (slot LEFT) -- the second half of mergeUnitaryFactor.  from_left:
// N . T over T's left bond (MPSTensor::multiply_from_left: T made right-paired,
// the product, the left index = N's left basis, back to left-paired); else T . N
// over its right bond (multiply_from_right: the right index = N's right basis).
// The left (right) index of the result keeps the sectors the new bond reaches, as
// the reference's MPSTensor constructor does.  OUT = the new tensor, left-paired.
qcm_plan* build_multiply(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& t, const BM& n,
                         bool from_left) {
    auto P = std::make_unique<qcm_plan>();
    P->kind = PK_MPS;
    int64_t len = 0;
    std::vector<Piece> ps;
    if (from_left) {
        BM rp = map_l2r(phys, left_i, right_i, t, QCM_BUF_KET, ps);
        add_map(P.get(), ps, rp, QCM_BUF_S0, len);
        P->scratch[0] = len;
        BM prod;
        add_product(P.get(), n, QCM_BUF_LEFT, rp, QCM_BUF_S0, QCM_BUF_S1, prod, len);
        P->scratch[1] = len;
        Idx new_left = left_basis(prod);
        Idx right = right_i;
        Idx reach = index_product(phys, new_left);
        common_subset(right, reach);
        ps.clear();
        BM lp = map_r2l(phys, new_left, right, prod, QCM_BUF_S1, ps);
        add_map(P.get(), ps, lp, QCM_BUF_OUT, len);
        P->out_elems = len;
        P->out_bm = lp.b;
        P->out_left = new_left;
        P->out_right = right;
    } else {
        BM prod;
        add_product(P.get(), t, QCM_BUF_KET, n, QCM_BUF_LEFT, QCM_BUF_OUT, prod, len);
        P->out_elems = len;
        Idx new_right = right_basis(prod);
        Idx left = left_i;
        Idx reach = index_product(adjoin(phys), new_right);
        common_subset(left, reach);
        P->out_bm = prod.b;
        P->out_left = left;
        P->out_right = new_right;
    }
    P->out_phys = phys;
    return P.release();
}

// A site tensor between its two pairings (reshape_left_to_right / reshape_right_to_left,
// mp_tensors/reshapes.h): to_right: KET left-paired -> OUT right-paired; else KET
// right-paired -> OUT left-paired.  Same indices in and out.
qcm_plan* build_reshape(const Idx& phys, const Idx& left_i, const Idx& right_i, const BM& t, bool to_right) {
    auto P = std::make_unique<qcm_plan>();
    P->kind = PK_MPS;
    int64_t len = 0;
    std::vector<Piece> ps;
    BM out = to_right ? map_l2r(phys, left_i, right_i, t, QCM_BUF_KET, ps)
                      : map_r2l(phys, left_i, right_i, t, QCM_BUF_KET, ps);
    add_map(P.get(), ps, out, QCM_BUF_OUT, len);
    P->out_elems = len;
    P->out_bm = out.b;
    P->out_phys = phys;
    P->out_left = left_i;
    P->out_right = right_i;
    return P.release();
}

// Output blocks of a grouped product, created on first use; every block's
// segments are summed in the order they were added (one zero stage, then one
// grouped GEMM stage; blocks no segment writes stay zero).
namespace {
struct ProductOut {
    BM C;
    std::map<std::array<int32_t, 4>, std::vector<GemmSeg>> segs;
    double flops = 0.0;

    void add(Q lc, Q rc, int64_t rows, int64_t cols, const GemmSeg& s) {
        const size_t k = C.find(lc, rc);
        if (k == C.b.size()) {
            Blk nb;
            nb.lc = lc;
            nb.rc = rc;
            nb.rows = rows;
            nb.cols = cols;
            C.insert(nb);
        } else if (C.b[k].rows != rows || C.b[k].cols != cols) {
            throw std::runtime_error("block product: products of one output block differ in shape");
        }
        segs[{lc.n, lc.s, rc.n, rc.s}].push_back(s);
        flops += 2.0 * rows * cols * s.K;
    }

    qcm_plan* finish() {
        auto P = std::make_unique<qcm_plan>();
        P->kind = PK_MPS;
        const int64_t len = C.assign_offsets(0);
        P->stages.push_back(zero_stage(QCM_BUF_OUT, len));
        Stage g;
        g.kind = ST_GEMM;
        for (const Blk& c : C.b) {
            const auto& v = segs[{c.lc.n, c.lc.s, c.rc.n, c.rc.s}];
            if (v.empty() || c.rows == 0 || c.cols == 0) continue;
            GemmOut o;
            o.c_buf = QCM_BUF_OUT;
            o.c_off = c.off;
            o.ldc = c.rows;
            o.M = c.rows;
            o.N = c.cols;
            o.s_begin = (int64_t)g.gseg.size();
            for (const GemmSeg& x : v)
                if (x.K > 0) g.gseg.push_back(x);
            o.s_end = (int64_t)g.gseg.size();
            if (o.s_end > o.s_begin) g.gout.push_back(o);
        }
        if (!g.gout.empty()) P->stages.push_back(std::move(g));
        P->gemm_flops = flops;
        P->out_elems = len;
        P->out_bm = C.b;
        return P.release();
    }
};

GemmSeg seg(int32_t abuf, const Blk& a, bool ta, int32_t bbuf, const Blk& b, bool tb, int64_t K, double alpha) {
    GemmSeg s;
    s.a_buf = abuf;
    s.ta = ta ? 1 : 0;
    s.a_off = a.off;
    s.lda = a.rows;
    s.b_buf = bbuf;
    s.tb = tb ? 1 : 0;
    s.b_off = b.off;
    s.ldb = b.rows;
    s.K = K;
    s.alpha = alpha;
    return s;
}
}  // namespace

// The charge-matched product of two block matrices, op(A) op(B) with op a
// transpose where asked (block_matrix gemm, block_matrix/block_matrix_algorithms.h:
// 47-80, with transpose(), :118-128): every pair of blocks whose inner charges
// agree adds its product to the output block (left charge of op(A), right charge
// of op(B)).  A in slot KET, B in slot LEFT, the product in OUT (blocks in DualIndex
// order, through qcm_plan_out_tensor).  Pairs are taken in A's order, then B's.
qcm_plan* build_block_gemm(const BM& A, bool ta, const BM& B, bool tb) {
    ProductOut out;
    // op(B) blocks by their left charge, in B's order
    std::map<std::pair<int, int>, std::vector<size_t>> by_left;
    for (size_t k = 0; k < B.b.size(); ++k) {
        const Q l = tb ? B.b[k].rc : B.b[k].lc;
        by_left[{l.n, l.s}].push_back(k);
    }
    for (const Blk& a : A.b) {
        const Q al = ta ? a.rc : a.lc, ar = ta ? a.lc : a.rc;
        const int64_t am = ta ? a.cols : a.rows, ak = ta ? a.rows : a.cols;
        auto it = by_left.find({ar.n, ar.s});
        if (it == by_left.end()) continue;
        for (size_t kb : it->second) {
            const Blk& b = B.b[kb];
            const Q br = tb ? b.lc : b.rc;
            const int64_t bk = tb ? b.cols : b.rows, bn = tb ? b.rows : b.cols;
            if (ak != bk) throw std::runtime_error("block product: inner dimensions differ");
            out.add(al, br, am, bn, seg(QCM_BUF_KET, a, ta, QCM_BUF_LEFT, b, tb, ak, 1.0));
        }
    }
    return out.finish();
}

// The density matrix of the heev truncation (TwoSiteTensor::predict_split_l2r /
// _r2l, mp_tensors/twositetensor.hpp:184-297, and predict_new_state_l2r/r2l_sweep,
// contractions/common/prediction.hpp:19-125): rho = theta theta^T (l2r, theta
// left-paired) or theta^T theta (r2l, theta right-paired), theta in slot KET;
// with alpha != 0, plus alpha sum_b h_b h_b^T (l2r) or alpha sum_b h_b^T h_b (r2l)
// over the blocks of the boundary tensor product h (left/right_boundary_tensor_mpo,
// slot RIGHT): for every bond b, the pairs of h[b]'s blocks that share their right
// charge (l2r) or left charge (r2l), restricted to the output charges (ci, cj)
// that theta holds as a block, and added to rho(ci, cj), created if absent.
qcm_plan* build_density_matrix(const BM& theta, bool l2r, const std::vector<BM>* half, double alpha) {
    ProductOut out;
    if (l2r) {
        // rho(ci, cj) = sum over rc of theta(ci, rc) theta(cj, rc)^T, in the order of
        // theta's blocks and, for one rc, of decreasing cj
        std::map<std::pair<int, int>, std::vector<size_t>> by_right;
        for (size_t k = 0; k < theta.b.size(); ++k) by_right[{theta.b[k].rc.n, theta.b[k].rc.s}].push_back(k);
        for (const Blk& a : theta.b)
            for (size_t kb : by_right[{a.rc.n, a.rc.s}]) {
                const Blk& b = theta.b[kb];
                out.add(a.lc, b.lc, a.rows, b.rows, seg(QCM_BUF_KET, a, false, QCM_BUF_KET, b, true, a.cols, 1.0));
            }
    } else {
        // rho(ci, cj) = sum over lc of theta(lc, ci)^T theta(lc, cj): the transposed
        // blocks in their own order (decreasing (rc, lc)), then theta's with that lc
        std::vector<size_t> order(theta.b.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) {
            const Blk& a = theta.b[x];
            const Blk& b = theta.b[y];
            return a.rc > b.rc || (a.rc == b.rc && a.lc > b.lc);
        });
        for (size_t ka : order) {
            const Blk& a = theta.b[ka];
            for (size_t kb = theta.left_lower_bound(a.lc); kb < theta.b.size() && theta.b[kb].lc == a.lc; ++kb) {
                const Blk& b = theta.b[kb];
                out.add(a.rc, b.rc, a.cols, b.cols, seg(QCM_BUF_KET, a, true, QCM_BUF_KET, b, false, a.rows, 1.0));
            }
        }
    }
    if (alpha != 0.0 && half) {
        for (const BM& hb : *half) {
            // groups of blocks with one right (l2r) / left (r2l) charge, in order of first appearance
            std::vector<std::pair<Q, std::vector<size_t>>> groups;
            for (size_t k = 0; k < hb.b.size(); ++k) {
                const Q g = l2r ? hb.b[k].rc : hb.b[k].lc;
                auto it = std::find_if(groups.begin(), groups.end(), [&](const auto& x) { return x.first == g; });
                if (it == groups.end()) groups.push_back({g, {k}});
                else it->second.push_back(k);
            }
            for (const auto& grp : groups)
                for (size_t i : grp.second)
                    for (size_t j : grp.second) {
                        const Blk& vi = hb.b[i];
                        const Blk& vj = hb.b[j];
                        const Q ci = l2r ? vi.lc : vi.rc, cj = l2r ? vj.lc : vj.rc;
                        if (theta.find(ci, cj) == theta.b.size()) continue;
                        if (l2r)
                            out.add(ci, cj, vi.rows, vj.rows,
                                    seg(QCM_BUF_RIGHT, vi, false, QCM_BUF_RIGHT, vj, true, vi.cols, alpha));
                        else
                            out.add(ci, cj, vi.cols, vj.cols,
                                    seg(QCM_BUF_RIGHT, vi, true, QCM_BUF_RIGHT, vj, false, vi.rows, alpha));
                    }
        }
    }
    return out.finish();
}

}  // namespace qcm

using namespace qcm;

// true for the abelian group; throws on an unknown one
static bool check_symmetry(int32_t symmetry) { return abelian_symmetry(symmetry); }

static int mps_guard(const char* what, const std::function<qcm_plan*()>& f, qcm_plan** out) {
    if (!out) { set_error(std::string(what) + ": null output"); return QCM_E_INVALID; }
    *out = nullptr;
    try {
        *out = f();
        return QCM_OK;
    } catch (const std::exception& e) {
        set_error(std::string(what) + ": " + e.what());
        return QCM_E_INVALID;
    }
}

extern "C" {

int qcm_plan_two_site(const qcm_index_t* phys1, const qcm_index_t* a_left, const qcm_index_t* a_right,
                      const qcm_blocks_t* a, const qcm_index_t* phys2, const qcm_index_t* b_left,
                      const qcm_index_t* b_right, const qcm_blocks_t* b, int32_t symmetry, qcm_plan** plan) {
    return mps_guard("qcm_plan_two_site", [&] {
        return build_theta(read_index(phys1), read_index(a_left), read_index(a_right), read_blocks(a),
                           read_index(phys2), read_index(b_left), read_index(b_right), read_blocks(b),
                           check_symmetry(symmetry));
    }, plan);
}

int qcm_plan_split_theta(const qcm_index_t* phys1, const qcm_index_t* phys2, const qcm_index_t* left_i,
                         const qcm_index_t* right_i, const qcm_blocks_t* u, int32_t symmetry, qcm_plan** plan) {
    return mps_guard("qcm_plan_split_theta", [&] {
        return build_split(read_index(phys1), read_index(phys2), read_index(left_i), read_index(right_i),
                           read_blocks(u), check_symmetry(symmetry));
    }, plan);
}

int qcm_plan_split_assemble(const qcm_plan* split, const int64_t* u_off, const int64_t* vt_off, const int64_t* keep,
                            const double* S_host, const int64_t* s_off, int32_t l2r, qcm_plan** plan) {
    if (!split || split->kind != PK_SPLIT) { set_error("qcm_plan_split_assemble: not a split plan"); return QCM_E_STATE; }
    if (!u_off || !vt_off || !keep || !S_host || !s_off) {
        set_error("qcm_plan_split_assemble: null argument");
        return QCM_E_INVALID;
    }
    BM both;
    both.b = split->out_bm;
    std::vector<int64_t> kdim(both.b.size());
    for (size_t i = 0; i < both.b.size(); ++i) {
        kdim[i] = std::min(both.b[i].rows, both.b[i].cols);
        if (keep[i] < 0 || keep[i] > kdim[i]) {
            set_error("qcm_plan_split_assemble: keep count of block " + std::to_string(i) + " out of range");
            return QCM_E_RANGE;
        }
    }
    // the split plan stores (phys1, left, right) and phys2 is recovered from the reduced tensor's index
    return mps_guard("qcm_plan_split_assemble", [&] {
        return build_assemble(split->out_phys, split->out2_phys, split->out_left, split->out_right, both, u_off,
                              vt_off, kdim.data(), keep, S_host, s_off, l2r != 0);
    }, plan);
}

int qcm_plan_mps_multiply(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                          const qcm_blocks_t* t, const qcm_blocks_t* n, int32_t from_left, qcm_plan** plan) {
    return mps_guard("qcm_plan_mps_multiply", [&] {
        return build_multiply(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(t),
                              read_blocks(n), from_left != 0);
    }, plan);
}

int qcm_plan_mps_reshape(const qcm_index_t* phys, const qcm_index_t* left_i, const qcm_index_t* right_i,
                         const qcm_blocks_t* t, int32_t to_right, qcm_plan** plan) {
    return mps_guard("qcm_plan_mps_reshape", [&] {
        return build_reshape(read_index(phys), read_index(left_i), read_index(right_i), read_blocks(t),
                             to_right != 0);
    }, plan);
}

int qcm_plan_block_gemm(const qcm_blocks_t* a, int32_t ta, const qcm_blocks_t* b, int32_t tb, qcm_plan** plan) {
    return mps_guard("qcm_plan_block_gemm", [&] { return build_block_gemm(read_blocks(a), ta != 0, read_blocks(b), tb != 0); },
                     plan);
}

int qcm_plan_density_matrix(const qcm_blocks_t* theta, int32_t l2r, const qcm_boundary_t* half, double alpha,
                            qcm_plan** plan) {
    return mps_guard("qcm_plan_density_matrix", [&] {
        std::vector<BM> h;
        if (half && alpha != 0.0) h = read_boundary(half);
        return build_density_matrix(read_blocks(theta), l2r != 0, (half && alpha != 0.0) ? &h : nullptr, alpha);
    }, plan);
}

// Output tensors of an MPS-level plan: which = 0 (OUT) or 1 (the second output of
// an assembly plan, in S2).  Call with NULL arrays for the counts.
int qcm_plan_out_tensor(const qcm_plan* p, int32_t which, int32_t* nblocks, int32_t* q, int64_t* rows, int64_t* cols,
                        int64_t* off, int32_t* n_idx3, int32_t* idx_q, int64_t* idx_size) {
    if (!p || (p->kind != PK_THETA && p->kind != PK_SPLIT && p->kind != PK_ASSEMBLE && p->kind != PK_MPS)) {
        set_error("qcm_plan_out_tensor: not an MPS-level plan");
        return QCM_E_STATE;
    }
    if (which != 0 && !(which == 1 && p->kind == PK_ASSEMBLE)) {
        set_error("qcm_plan_out_tensor: no such output");
        return QCM_E_INVALID;
    }
    const auto& bm = which == 0 ? p->out_bm : p->out2_bm;
    const Idx* ix[3] = {which == 0 ? &p->out_phys : &p->out2_phys, which == 0 ? &p->out_left : &p->out2_left,
                        which == 0 ? &p->out_right : &p->out2_right};
    if (nblocks) *nblocks = (int32_t)bm.size();
    for (size_t k = 0; k < bm.size(); ++k) {
        if (q) {
            q[4 * k] = bm[k].lc.n;
            q[4 * k + 1] = bm[k].lc.s;
            q[4 * k + 2] = bm[k].rc.n;
            q[4 * k + 3] = bm[k].rc.s;
        }
        if (rows) rows[k] = bm[k].rows;
        if (cols) cols[k] = bm[k].cols;
        if (off) off[k] = bm[k].off;
    }
    int64_t base = 0;
    for (int i = 0; i < 3; ++i) {
        if (n_idx3) n_idx3[i] = (int32_t)ix[i]->d.size();
        for (size_t k = 0; k < ix[i]->d.size(); ++k) {
            if (idx_q) {
                idx_q[2 * (base + k)] = ix[i]->d[k].first.n;
                idx_q[2 * (base + k) + 1] = ix[i]->d[k].first.s;
            }
            if (idx_size) idx_size[base + k] = ix[i]->d[k].second;
        }
        base += (int64_t)ix[i]->d.size();
    }
    return QCM_OK;
}

}  // extern "C"
