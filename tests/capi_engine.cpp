// The two-site microiteration of tests/capi_microiteration.cpp written against
// the reference-facing C++ classes (include/qcm_gb300_engine.hpp) instead of
// the raw C ABI -- the shape QCMaquis's own sweep code has (one step of
// sba/SweepBasedEnergyMinimization.h:75-140):
//
//   TwoSiteTensor tst(mps[i], mps[i+1]);
//   SiteProblem sp(left[i], right[i+2], ts_mpo[i]);
//   auto res = solve_ietl_jcd(sp, tst.make_mps(), parms);
//   tst << res.second;
//   boost::tie(mps[i], mps[i+1], trunc) = tst.split_mps_l2r(Mmax, cutoff);
//   left[i+1] = contr::overlap_mpo_left_step(mps[i], mps[i], left[i], mpo[i]);
//
// Same inputs and outputs as capi_microiteration (file format: capi_io.hpp).
#include <cstdio>
#include <string>
#include <vector>

#include "qcm_gb300_engine.hpp"
#include "capi_io.hpp"

using namespace capi_io;

namespace {

qcm::IndexArr index_of(Inputs& in, const std::string& k) {
    qcm::IndexArr x;
    const int64_t n = in.n(k + ".size");
    x.q.assign(in.p<int32_t>(k + ".q"), in.p<int32_t>(k + ".q") + 2 * n);
    x.size.assign(in.p<int64_t>(k + ".size"), in.p<int64_t>(k + ".size") + n);
    return x;
}

qcm::Blocks blocks_of(Inputs& in, const std::string& k) {
    qcm::Blocks b;
    const int64_t n = in.n(k + ".rows");
    b.q.assign(in.p<int32_t>(k + ".q"), in.p<int32_t>(k + ".q") + 4 * n);
    b.rows.assign(in.p<int64_t>(k + ".rows"), in.p<int64_t>(k + ".rows") + n);
    b.cols.assign(in.p<int64_t>(k + ".cols"), in.p<int64_t>(k + ".cols") + n);
    b.off.assign(in.p<int64_t>(k + ".off"), in.p<int64_t>(k + ".off") + n);
    return b;
}

qcm::MPSTensor tensor_of(Inputs& in, const std::string& k) {
    qcm::MPSTensor t;
    t.phys = index_of(in, "phys");
    t.left = index_of(in, k + ".left");
    t.right = index_of(in, k + ".right");
    t.blocks = blocks_of(in, k);
    t.data = qcm::DeviceArray::from_host(in.p<double>(k + ".data"), in.n(k + ".data"));
    return t;
}

qcm::Boundary boundary_of(Inputs& in, const std::string& k) {
    qcm::Boundary b;
    const int64_t nb = in.n(k + ".blk_ptr");
    b.blk_ptr.assign(in.p<int32_t>(k + ".blk_ptr"), in.p<int32_t>(k + ".blk_ptr") + nb);
    b.blocks = blocks_of(in, k);
    b.data = qcm::DeviceArray::from_host(in.p<double>(k + ".data"), in.n(k + ".data"));
    return b;
}

void put_tensor(Writer& out, const std::string& k, const qcm::MPSTensor& t) {
    const std::vector<double> h = t.data.to_host();
    out.put(k + ".q", 'i', t.blocks.q.data(), (int64_t)t.blocks.q.size());
    out.put(k + ".rows", 'l', t.blocks.rows.data(), (int64_t)t.blocks.rows.size());
    out.put(k + ".cols", 'l', t.blocks.cols.data(), (int64_t)t.blocks.cols.size());
    out.put(k + ".data", 'd', h.data(), (int64_t)h.size());
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s inputs.bin outputs.bin\n", argv[0]);
        return 2;
    }
    try {
        Inputs in{read_arrays(argv[1])};
        qcm::Engine engine;
        const qcm::MPSTensor A = tensor_of(in, "A"), B = tensor_of(in, "B");
        const qcm::Boundary L = boundary_of(in, "L"), R = boundary_of(in, "R");
        const qcm_mpo_t ts = in.mpo("ts"), w = in.mpo("W");

        qcm::TwoSiteTensor tst(engine, A, B);
        const qcm::SiteProblem sp{L, R, ts};
        int iters = 0;
        auto res = qcm::solve_ietl_jcd(engine, sp, tst.make_mps(), in.d("tol"), (int)in.d("maxiter"), {},
                                       QCM_PREC_FP64, &iters);
        tst << res.second;
        auto [A2, B2, tr] = tst.split_mps_l2r((int64_t)in.d("Mmax"), in.d("cutoff"));
        const qcm::Boundary L2 = engine.overlap_mpo_left_step(A2, L, w);

        const std::vector<double> hL2 = L2.data.to_host();
        Writer out(argv[2]);
        const double scal[5] = {res.first, tr.truncated_weight, tr.truncated_fraction, tr.smallest_ev,
                                (double)tr.bond_dimension};
        out.put("scalars", 'd', scal, 5);
        const int32_t it32 = iters;
        out.put("iters", 'i', &it32, 1);
        out.put("L2.blk_ptr", 'i', L2.blk_ptr.data(), (int64_t)L2.blk_ptr.size());
        out.put("L2.q", 'i', L2.blocks.q.data(), (int64_t)L2.blocks.q.size());
        out.put("L2.rows", 'l', L2.blocks.rows.data(), (int64_t)L2.blocks.rows.size());
        out.put("L2.cols", 'l', L2.blocks.cols.data(), (int64_t)L2.blocks.cols.size());
        out.put("L2.off", 'l', L2.blocks.off.data(), (int64_t)L2.blocks.off.size());
        out.put("L2.data", 'd', hL2.data(), (int64_t)hL2.size());
        put_tensor(out, "A2", A2);
        put_tensor(out, "B2", B2);
        std::printf("energy %.15f iterations %d bond %lld weight %.3e\n", res.first, iters,
                    (long long)tr.bond_dimension, tr.truncated_weight);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
