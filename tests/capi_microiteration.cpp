// One two-site DMRG microiteration driven from C++ through the C ABI only, the
// way a C++ host (QCMaquis's SweepBasedEnergyMinimization, one step of
// sba/GenericSweepSimulation.h:73-152) would drive it:
//   TwoSiteTensor(mps[i], mps[i+1])  -> qcm_plan_two_site + qcm_ctx_run
//   solve_ietl_jcd                   -> qcm_plan_sigma + qcm_jcd_solve
//   split_mps_l2r                    -> qcm_split
//   updateLeftBoundary               -> qcm_plan_boundary_left + qcm_boundary_step
// Inputs (site tensors, boundaries, MPO tensors, parameters) come from a file of
// named arrays written by the test; outputs (energy, truncation results, the new
// left boundary and the new site tensors) go to another such file.
// The file format is in tests/capi_io.hpp.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <stdexcept>
#include <string>
#include <vector>

#include "qcm_gb300.h"
#include "capi_io.hpp"

using namespace capi_io;

namespace {

// an index / block list read back from the library (owning arrays)
struct Tensor {
    std::vector<int32_t> bq, iq;
    std::vector<int64_t> rows, cols, off, isz;
    int32_t n3[3] = {0, 0, 0};
    qcm_index_t idx(int i) const {
        int64_t base = 0;
        for (int k = 0; k < i; ++k) base += n3[k];
        return {n3[i], iq.data() + 2 * base, isz.data() + base};
    }
    qcm_blocks_t blocks() const {
        return {(int32_t)rows.size(), bq.data(), rows.data(), cols.data(), off.data()};
    }
    int64_t elems() const {
        int64_t e = 0;
        for (size_t k = 0; k < rows.size(); ++k) e = std::max<int64_t>(e, off[k] + rows[k] * cols[k]);
        return e;
    }
};

template <class F>
Tensor read_tensor(F query) {
    Tensor t;
    int32_t nb = 0;
    ok(query(&nb, nullptr, nullptr, nullptr, nullptr, t.n3, nullptr, nullptr), "tensor query");
    t.bq.resize(4 * (size_t)std::max(nb, 1));
    t.rows.resize(nb);
    t.cols.resize(nb);
    t.off.resize(nb);
    const int32_t ni = t.n3[0] + t.n3[1] + t.n3[2];
    t.iq.resize(2 * (size_t)std::max(ni, 1));
    t.isz.resize(std::max(ni, 1));
    ok(query(&nb, t.bq.data(), t.rows.data(), t.cols.data(), t.off.data(), t.n3, t.iq.data(), t.isz.data()),
       "tensor query");
    return t;
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 3) {
        std::fprintf(stderr, "usage: %s inputs.bin outputs.bin\n", argv[0]);
        return 2;
    }
    try {
        Inputs in{read_arrays(argv[1])};
        qcm_ctx* ctx = nullptr;
        ok(qcm_ctx_create(nullptr, &ctx), "qcm_ctx_create");
        qcm_index_t phys = in.index("phys");
        // TwoSiteTensor(mps[i], mps[i+1]).make_mps()
        qcm_plan* tp = nullptr;
        qcm_index_t al = in.index("A.left"), ar = in.index("A.right"), bl = in.index("B.left"),
                    br = in.index("B.right");
        qcm_blocks_t ab = in.blocks("A"), bb = in.blocks("B");
        ok(qcm_plan_two_site(&phys, &al, &ar, &ab, &phys, &bl, &br, &bb, QCM_SYM_SU2U1, &tp), "qcm_plan_two_site");
        Tensor psi = read_tensor([&](int32_t* nb, int32_t* q, int64_t* r, int64_t* c, int64_t* o, int32_t* n3,
                                     int32_t* iq, int64_t* is) {
            return qcm_plan_out_tensor(tp, 0, nb, q, r, c, o, n3, iq, is);
        });
        double* dA = in.device("A.data");
        double* dB = in.device("B.data");
        double* dpsi = nullptr;
        const int64_t n = psi.elems();
        cudaMalloc(&dpsi, sizeof(double) * n);
        ok(qcm_ctx_run(ctx, tp, dA, dB, 0, nullptr, 0, dpsi, QCM_PREC_FP64), "two-site tensor");
        // solve_ietl_jcd on SiteProblem(L[i], R[i+2], ts_mpo[i])
        qcm_boundary_t L = in.boundary("L"), R = in.boundary("R");
        qcm_mpo_t ts = in.mpo("ts"), w = in.mpo("W");
        double* dL = in.device("L.data");
        double* dR = in.device("R.data");
        qcm_plan* sp = nullptr;
        qcm_index_t p2 = psi.idx(0), pl = psi.idx(1), pr = psi.idx(2);
        qcm_blocks_t pb = psi.blocks();
        ok(qcm_plan_sigma(&p2, &pl, &pr, &pb, &L, &R, &ts, 1, &sp), "qcm_plan_sigma");
        double* du = nullptr;
        cudaMalloc(&du, sizeof(double) * n);
        double energy = 0.0;
        int32_t iters = 0;
        ok(qcm_jcd_solve(ctx, sp, dL, in.n("L.data"), dR, in.n("R.data"), QCM_PREC_FP64, dpsi, n, in.d("tol"),
                         (int32_t)in.d("maxiter"), nullptr, 0, du, &energy, &iters), "qcm_jcd_solve");
        // split_mps_l2r(Mmax, cutoff)
        qcm_trunc_t tr;
        qcm_split_result* res = nullptr;
        ok(qcm_split(ctx, &phys, &phys, &al, &br, &pb, du, 1, (int64_t)in.d("Mmax"), in.d("cutoff"), QCM_SYM_SU2U1, &tr,
                     &res),
           "qcm_split");
        const double* dA2 = nullptr;
        const double* dB2 = nullptr;
        Tensor A2 = read_tensor([&](int32_t* nb, int32_t* q, int64_t* r, int64_t* c, int64_t* o, int32_t* n3,
                                    int32_t* iq, int64_t* is) {
            return qcm_split_result_tensor(res, 0, nb, q, r, c, o, n3, iq, is, &dA2);
        });
        Tensor B2 = read_tensor([&](int32_t* nb, int32_t* q, int64_t* r, int64_t* c, int64_t* o, int32_t* n3,
                                    int32_t* iq, int64_t* is) {
            return qcm_split_result_tensor(res, 1, nb, q, r, c, o, n3, iq, is, &dB2);
        });
        // L[i+1] = overlap_mpo_left_step(A', A', L[i], W[i])
        qcm_plan* bp = nullptr;
        qcm_index_t a2p = A2.idx(0), a2l = A2.idx(1), a2r = A2.idx(2);
        qcm_blocks_t a2b = A2.blocks();
        ok(qcm_plan_boundary_left(&a2p, &a2l, &a2r, &a2b, &L, &w, 1, &bp), "qcm_plan_boundary_left");
        int32_t aux = 0, nbl = 0;
        ok(qcm_plan_out_layout(bp, &aux, &nbl, nullptr, nullptr, nullptr, nullptr, nullptr), "qcm_plan_out_layout");
        std::vector<int32_t> lptr(aux + 1), lq(4 * (size_t)std::max(nbl, 1));
        std::vector<int64_t> lrows(std::max(nbl, 1)), lcols(std::max(nbl, 1)), loff(std::max(nbl, 1));
        ok(qcm_plan_out_layout(bp, &aux, &nbl, lptr.data(), lq.data(), lrows.data(), lcols.data(), loff.data()),
           "qcm_plan_out_layout");
        int64_t lsize = 0;
        for (int k = 0; k < nbl; ++k) lsize = std::max<int64_t>(lsize, loff[k] + lrows[k] * lcols[k]);
        double* dL2 = nullptr;
        cudaMalloc(&dL2, sizeof(double) * std::max<int64_t>(lsize, 1));
        ok(qcm_boundary_step(ctx, bp, dA2, dL, in.n("L.data"), dL2, QCM_PREC_FP64), "qcm_boundary_step");
        std::vector<double> hL2(lsize), hA2(A2.elems()), hB2(B2.elems());
        cudaMemcpy(hL2.data(), dL2, sizeof(double) * lsize, cudaMemcpyDeviceToHost);
        cudaMemcpy(hA2.data(), dA2, sizeof(double) * hA2.size(), cudaMemcpyDeviceToHost);
        cudaMemcpy(hB2.data(), dB2, sizeof(double) * hB2.size(), cudaMemcpyDeviceToHost);
        if (cudaDeviceSynchronize() != cudaSuccess) throw std::runtime_error("device error");
        Writer out(argv[2]);
        const double scal[5] = {energy, tr.truncated_weight, tr.truncated_fraction, tr.smallest_ev,
                                (double)tr.bond_dimension};
        out.put("scalars", 'd', scal, 5);
        out.put("iters", 'i', &iters, 1);
        out.put("L2.blk_ptr", 'i', lptr.data(), aux + 1);
        out.put("L2.q", 'i', lq.data(), 4 * (int64_t)nbl);
        out.put("L2.rows", 'l', lrows.data(), nbl);
        out.put("L2.cols", 'l', lcols.data(), nbl);
        out.put("L2.off", 'l', loff.data(), nbl);
        out.put("L2.data", 'd', hL2.data(), lsize);
        out.put("A2.q", 'i', A2.bq.data(), 4 * (int64_t)A2.rows.size());
        out.put("A2.rows", 'l', A2.rows.data(), (int64_t)A2.rows.size());
        out.put("A2.cols", 'l', A2.cols.data(), (int64_t)A2.cols.size());
        out.put("A2.data", 'd', hA2.data(), (int64_t)hA2.size());
        out.put("B2.q", 'i', B2.bq.data(), 4 * (int64_t)B2.rows.size());
        out.put("B2.rows", 'l', B2.rows.data(), (int64_t)B2.rows.size());
        out.put("B2.cols", 'l', B2.cols.data(), (int64_t)B2.cols.size());
        out.put("B2.data", 'd', hB2.data(), (int64_t)hB2.size());
        std::printf("energy %.15f iterations %d bond %lld weight %.3e\n", energy, iters,
                    (long long)tr.bond_dimension, tr.truncated_weight);
        qcm_split_result_destroy(res);
        qcm_plan_destroy(tp);
        qcm_plan_destroy(sp);
        qcm_plan_destroy(bp);
        cudaFree(dA); cudaFree(dB); cudaFree(dpsi); cudaFree(du); cudaFree(dL); cudaFree(dR); cudaFree(dL2);
        qcm_ctx_destroy(ctx);
    } catch (const std::exception& e) {
        std::fprintf(stderr, "error: %s\n", e.what());
        return 1;
    }
    return 0;
}
