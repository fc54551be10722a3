// qcm_gb300.hpp -- header-only C++ layer over the C ABI in qcm_gb300.h.
//
// Mirrors the calling pattern of contraction::Engine<..., SU2U1>
// (dmrg/framework/dmrg/mp_tensors/contractions/non-abelian/engine.hpp:104-207):
// build a plan for (layouts, MPO tensor) once, run it on device buffers as
// many times as the eigensolver needs.  Errors become qcm::error exceptions,
// as the reference throws std::runtime_error.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

#include "qcm_gb300.h"

namespace qcm {

struct error : std::runtime_error {
    int code;
    error(int c, const std::string& what) : std::runtime_error(what), code(c) {}
};

inline void check(int rc, const char* what) {
    if (rc != QCM_OK) throw error(rc, std::string(what) + ": " + qcm_last_error());
}

// Owning view of one block list (charges (N,2S), shapes, element offsets).
struct Blocks {
    std::vector<int32_t> q;
    std::vector<int64_t> rows, cols, off;
    void add(int ln, int l2s, int rn, int r2s, int64_t r, int64_t c) {
        q.insert(q.end(), {ln, l2s, rn, r2s});
        off.push_back(size());
        rows.push_back(r);
        cols.push_back(c);
    }
    int64_t size() const {
        int64_t s = 0;
        for (size_t k = 0; k < rows.size(); ++k) s = std::max(s, off[k] + rows[k] * cols[k]);
        return s;
    }
    qcm_blocks_t view() const {
        return qcm_blocks_t{(int32_t)rows.size(), q.data(), rows.data(), cols.data(), off.data()};
    }
};

struct IndexArr {
    std::vector<int32_t> q;
    std::vector<int64_t> size;
    void add(int n, int twoS, int64_t s) {
        q.insert(q.end(), {n, twoS});
        size.push_back(s);
    }
    qcm_index_t view() const { return qcm_index_t{(int32_t)size.size(), q.data(), size.data()}; }
};

class Plan {
public:
    explicit Plan(qcm_plan* p) : p_(p) {}
    Plan(Plan&& o) noexcept : p_(std::exchange(o.p_, nullptr)) {}
    Plan& operator=(Plan&& o) noexcept {
        if (this != &o) { reset(); p_ = std::exchange(o.p_, nullptr); }
        return *this;
    }
    Plan(const Plan&) = delete;
    Plan& operator=(const Plan&) = delete;
    ~Plan() { reset(); }

    qcm_plan* get() const { return p_; }

    int64_t out_elems() const {
        int64_t o = 0, s[3];
        check(qcm_plan_sizes(p_, &o, s), "qcm_plan_sizes");
        return o;
    }
    std::vector<int64_t> scratch_elems() const {
        int64_t o = 0, s[3];
        check(qcm_plan_sizes(p_, &o, s), "qcm_plan_sizes");
        return {s[0], s[1], s[2]};
    }
    double gemm_flops() const {
        double g = 0, a = 0, b = 0;
        int32_t n = 0;
        check(qcm_plan_work(p_, &g, &a, &b, &n), "qcm_plan_work");
        return g;
    }
    void upload() { check(qcm_plan_upload(p_), "qcm_plan_upload"); }
    // bufs: KET, LEFT, RIGHT, OUT, S0, S1, S2 device pointers
    void run(double* const bufs[QCM_NBUF], int precision = QCM_PREC_FP64, void* stream = nullptr) {
        check(qcm_plan_run(p_, bufs, precision, stream), "qcm_plan_run");
    }

private:
    void reset() {
        if (p_) qcm_plan_destroy(p_);
        p_ = nullptr;
    }
    qcm_plan* p_ = nullptr;
};

// Engine::site_hamil2 analogue: plan for sigma = H_eff psi.
inline Plan plan_site_hamil2(const qcm_index_t& phys, const qcm_index_t& left_i, const qcm_index_t& right_i,
                             const qcm_blocks_t& psi, const qcm_boundary_t& left, const qcm_boundary_t& right,
                             const qcm_mpo_t& mpo, bool hermitian = true) {
    qcm_plan* p = nullptr;
    check(qcm_plan_sigma(&phys, &left_i, &right_i, &psi, &left, &right, &mpo, hermitian ? 1 : 0, &p),
          "qcm_plan_sigma");
    return Plan(p);
}

// Engine::overlap_mpo_left_step / overlap_mpo_right_step analogues.
inline Plan plan_overlap_mpo_left_step(const qcm_index_t& phys, const qcm_index_t& left_i,
                                       const qcm_index_t& right_i, const qcm_blocks_t& mps,
                                       const qcm_boundary_t& left, const qcm_mpo_t& mpo, bool hermitian = true) {
    qcm_plan* p = nullptr;
    check(qcm_plan_boundary_left(&phys, &left_i, &right_i, &mps, &left, &mpo, hermitian ? 1 : 0, &p),
          "qcm_plan_boundary_left");
    return Plan(p);
}

inline Plan plan_overlap_mpo_right_step(const qcm_index_t& phys, const qcm_index_t& left_i,
                                        const qcm_index_t& right_i, const qcm_blocks_t& mps,
                                        const qcm_boundary_t& right, const qcm_mpo_t& mpo, bool hermitian = true) {
    qcm_plan* p = nullptr;
    check(qcm_plan_boundary_right(&phys, &left_i, &right_i, &mps, &right, &mpo, hermitian ? 1 : 0, &p),
          "qcm_plan_boundary_right");
    return Plan(p);
}

}  // namespace qcm
