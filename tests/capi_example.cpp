// Builds a sigma plan through the C++ layer over the C ABI for the smallest
// SU2U1 problem: one site pair with N=2, S=0 (two electrons in two orbitals),
// a 1x1 left and right boundary, and a one-element MPO carrying the two-site
// identity.  Prints the plan sizes; no GPU is needed to build a plan.
#include <cstdio>

#include "qcm_gb300.hpp"

int main() {
    qcm::IndexArr phys, left, right;
    // two-site reduced physical basis containing the (2,0) sector of size 4
    phys.add(2, 0, 4);
    left.add(0, 0, 1);
    right.add(2, 0, 1);
    qcm::Blocks psi;  // left-paired: rows (phys x left) = 4, cols = 1
    psi.add(2, 0, 2, 0, 4, 1);
    // boundaries: one bond index, one 1x1 block each
    int32_t lptr[2] = {0, 1}, rptr[2] = {0, 1};
    int32_t lq[4] = {0, 0, 0, 0}, rq[4] = {2, 0, 2, 0};
    int64_t one[1] = {1}, zero[1] = {0};
    qcm_boundary_t L{1, lptr, lq, one, one, zero}, R{1, rptr, rq, one, one, zero};
    // MPO: a single element (0,0) with one operator: identity on the (2,0) sector (4x4, diagonal)
    int32_t spin0[1] = {0}, herm0[1] = {0}, phase1[1] = {1};
    int32_t col_ptr[2] = {0, 1}, row_of[1] = {0}, term_ptr[2] = {0, 1}, term_op[1] = {0};
    double term_scale[1] = {1.0};
    int32_t op_spin[1] = {0}, op_blk_ptr[2] = {0, 1}, blk_q[4] = {2, 0, 2, 0}, blk_ent_ptr[2] = {0, 4};
    int32_t ent[16] = {0, 0, 0, 0, 1, 1, 0, 0, 2, 2, 0, 0, 3, 3, 0, 0};
    double ent_coeff[4] = {1.0, 1.0, 1.0, 1.0};
    qcm_mpo_t W{1, 1, spin0, spin0, herm0, herm0, phase1, phase1, col_ptr, row_of, term_ptr, term_op, term_scale,
                1, op_spin, op_blk_ptr, blk_q, blk_ent_ptr, ent, ent_coeff};
    try {
        qcm::Plan p = qcm::plan_site_hamil2(phys.view(), left.view(), right.view(), psi.view(), L, R, W);
        auto sc = p.scratch_elems();
        std::printf("out=%lld scratch=%lld,%lld,%lld gemm_flops=%.0f\n", (long long)p.out_elems(),
                    (long long)sc[0], (long long)sc[1], (long long)sc[2], p.gemm_flops());
    } catch (const qcm::error& e) {
        std::printf("error %d: %s\n", e.code, e.what());
        return 1;
    }
    return 0;
}
