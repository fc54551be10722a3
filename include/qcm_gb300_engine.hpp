// qcm_gb300_engine.hpp -- the reference-facing C++ classes of the two-site step,
// header-only, over the C ABI in qcm_gb300.h.
//
// A C++ host written against QCMaquis's surfaces finds them here under the
// same names and with the same meaning, the tensors living on the GPU:
//
//   MPSTensor       mp_tensors/mpstensor.h:30-142   indices, left-paired blocks, FP64 data
//   Boundary        mp_tensors/boundary.h:21-145    one block list per MPO bond, one arena
//   Engine          contractions/non-abelian/engine.hpp:84-226
//                   site_hamil2, overlap_mpo_left_step, overlap_mpo_right_step
//   SiteProblem     mp_tensors/siteproblem.h:22-53
//   solve_ietl_jcd  optimize/ietl_jacobi_davidson.h:16-77
//   TwoSiteTensor   mp_tensors/twositetensor.h:25-102   make_mps, operator<<,
//                   split_mps_l2r, split_mps_r2l
//
// (paths inside dmrg/framework/dmrg/).  MPO tensors are passed as qcm_mpo_t
// views of the caller's arrays.  Every call runs on the Engine's context
// (qcm_ctx: its stream, scratch and eigensolver workspace); plans are built for
// each call and released when it returns (the library frees their tables in
// stream order).  Errors become qcm::error exceptions, as the reference throws
// std::runtime_error.  Needs the CUDA runtime (device arrays are cudaMalloc'd).
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "qcm_gb300.hpp"

namespace qcm {

inline void cuda_check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw error(QCM_E_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

// FP64 device array, owned.
class DeviceArray {
public:
    DeviceArray() = default;
    explicit DeviceArray(int64_t n) : n_(n) {
        cuda_check(cudaMalloc(reinterpret_cast<void**>(&p_), sizeof(double) * (size_t)std::max<int64_t>(n, 1)),
                   "cudaMalloc");
    }
    DeviceArray(DeviceArray&& o) noexcept : p_(std::exchange(o.p_, nullptr)), n_(std::exchange(o.n_, 0)) {}
    DeviceArray& operator=(DeviceArray&& o) noexcept {
        if (this != &o) {
            reset();
            p_ = std::exchange(o.p_, nullptr);
            n_ = std::exchange(o.n_, 0);
        }
        return *this;
    }
    DeviceArray(const DeviceArray&) = delete;
    DeviceArray& operator=(const DeviceArray&) = delete;
    ~DeviceArray() { reset(); }

    static DeviceArray from_host(const double* h, int64_t n) {
        DeviceArray a(n);
        if (n > 0) cuda_check(cudaMemcpy(a.p_, h, sizeof(double) * n, cudaMemcpyHostToDevice), "cudaMemcpy");
        return a;
    }
    static DeviceArray copy_of(const double* d, int64_t n, cudaStream_t s) {
        DeviceArray a(n);
        if (n > 0)
            cuda_check(cudaMemcpyAsync(a.p_, d, sizeof(double) * n, cudaMemcpyDeviceToDevice, s), "cudaMemcpyAsync");
        return a;
    }
    std::vector<double> to_host(cudaStream_t s = nullptr) const {
        std::vector<double> h((size_t)n_);
        if (n_ > 0) {
            cuda_check(cudaMemcpyAsync(h.data(), p_, sizeof(double) * n_, cudaMemcpyDeviceToHost, s),
                       "cudaMemcpyAsync");
            cuda_check(cudaStreamSynchronize(s), "cudaStreamSynchronize");
        }
        return h;
    }
    double* get() { return p_; }
    const double* get() const { return p_; }
    int64_t size() const { return n_; }

private:
    void reset() {
        if (p_) cudaFree(p_);
        p_ = nullptr;
        n_ = 0;
    }
    double* p_ = nullptr;
    int64_t n_ = 0;
};

// MPSTensor on the device: physical, left and right indices, the left-paired
// blocks in DualIndex order (element offsets into data), FP64 data.
struct MPSTensor {
    IndexArr phys, left, right;
    Blocks blocks;
    DeviceArray data;
    int64_t elems() const { return blocks.size(); }
};

// Boundary on the device: the block lists of all MPO bonds b, bond b owning
// blocks [blk_ptr[b], blk_ptr[b+1]), offsets into one arena.
struct Boundary {
    std::vector<int32_t> blk_ptr{0};
    Blocks blocks;
    DeviceArray data;
    int32_t aux() const { return (int32_t)blk_ptr.size() - 1; }
    int64_t elems() const { return blocks.size(); }
    qcm_boundary_t view() const {
        return qcm_boundary_t{aux(), blk_ptr.data(), blocks.q.data(), blocks.rows.data(), blocks.cols.data(),
                              blocks.off.data()};
    }
};

namespace detail {

// layout and indices of a tensor the library describes (qcm_plan_out_tensor /
// qcm_split_result_tensor calling convention: counts first, then the arrays)
template <class Query>
void read_tensor_layout(Query query, MPSTensor& t) {
    int32_t nb = 0, n3[3] = {0, 0, 0};
    check(query(&nb, nullptr, nullptr, nullptr, nullptr, n3, nullptr, nullptr), "tensor layout");
    const int32_t ni = n3[0] + n3[1] + n3[2];
    std::vector<int32_t> q(4 * (size_t)std::max(nb, 1)), iq(2 * (size_t)std::max(ni, 1));
    std::vector<int64_t> r((size_t)std::max(nb, 1)), c((size_t)std::max(nb, 1)), o((size_t)std::max(nb, 1)),
        isz((size_t)std::max(ni, 1));
    check(query(&nb, q.data(), r.data(), c.data(), o.data(), n3, iq.data(), isz.data()), "tensor layout");
    t.blocks.q.assign(q.begin(), q.begin() + 4 * (size_t)nb);
    t.blocks.rows.assign(r.begin(), r.begin() + nb);
    t.blocks.cols.assign(c.begin(), c.begin() + nb);
    t.blocks.off.assign(o.begin(), o.begin() + nb);
    IndexArr* ix[3] = {&t.phys, &t.left, &t.right};
    int64_t base = 0;
    for (int i = 0; i < 3; ++i) {
        ix[i]->q.assign(iq.begin() + 2 * base, iq.begin() + 2 * (base + n3[i]));
        ix[i]->size.assign(isz.begin() + base, isz.begin() + base + n3[i]);
        base += n3[i];
    }
}

// a tensor with t's indices and layout and fresh data
inline MPSTensor like(const MPSTensor& t) {
    MPSTensor o;
    o.phys = t.phys;
    o.left = t.left;
    o.right = t.right;
    o.blocks = t.blocks;
    o.data = DeviceArray(t.elems());
    return o;
}

}  // namespace detail

// contraction::Engine: the contractions of the two-site step on one context.
class Engine {
public:
    explicit Engine(cudaStream_t stream = nullptr, bool hermitian = true) : stream_(stream), herm_(hermitian) {
        check(qcm_ctx_create(stream, &ctx_), "qcm_ctx_create");
    }
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;
    ~Engine() {
        if (ctx_) qcm_ctx_destroy(ctx_);
    }
    qcm_ctx* ctx() const { return ctx_; }
    cudaStream_t stream() const { return stream_; }
    bool hermitian() const { return herm_; }

    // the sigma plan of a site problem (kept by callers that apply it many times)
    Plan sigma_plan(const MPSTensor& ket, const Boundary& left, const Boundary& right, const qcm_mpo_t& mpo) const {
        const qcm_index_t p = ket.phys.view(), l = ket.left.view(), r = ket.right.view();
        const qcm_blocks_t b = ket.blocks.view();
        const qcm_boundary_t L = left.view(), R = right.view();
        return plan_site_hamil2(p, l, r, b, L, R, mpo, herm_);
    }

    // Engine::site_hamil2: sigma = H_eff ket
    MPSTensor site_hamil2(const MPSTensor& ket, const Boundary& left, const Boundary& right, const qcm_mpo_t& mpo,
                          int precision = QCM_PREC_FP64) {
        Plan p = sigma_plan(ket, left, right, mpo);
        MPSTensor out = detail::like(ket);
        check(qcm_ctx_run(ctx_, p.get(), ket.data.get(), left.data.get(), left.elems(), right.data.get(),
                          right.elems(), out.data.get(), precision),
              "site_hamil2");
        return out;
    }

    // Engine::overlap_mpo_left_step(bra = ket, ket, L[i], W[i]) -> L[i+1]
    Boundary overlap_mpo_left_step(const MPSTensor& ket, const Boundary& left, const qcm_mpo_t& mpo) {
        return boundary_step(true, ket, left, mpo);
    }
    // Engine::overlap_mpo_right_step(bra = ket, ket, R[i+1], W[i]) -> R[i]
    Boundary overlap_mpo_right_step(const MPSTensor& ket, const Boundary& right, const qcm_mpo_t& mpo) {
        return boundary_step(false, ket, right, mpo);
    }

private:
    Boundary boundary_step(bool to_right, const MPSTensor& ket, const Boundary& b, const qcm_mpo_t& mpo) {
        const qcm_index_t p = ket.phys.view(), l = ket.left.view(), r = ket.right.view();
        const qcm_blocks_t kb = ket.blocks.view();
        const qcm_boundary_t bv = b.view();
        Plan plan = to_right ? plan_overlap_mpo_left_step(p, l, r, kb, bv, mpo, herm_)
                             : plan_overlap_mpo_right_step(p, l, r, kb, bv, mpo, herm_);
        Boundary out;
        int32_t aux = 0, nb = 0;
        check(qcm_plan_out_layout(plan.get(), &aux, &nb, nullptr, nullptr, nullptr, nullptr, nullptr),
              "qcm_plan_out_layout");
        out.blk_ptr.assign((size_t)aux + 1, 0);
        out.blocks.q.assign(4 * (size_t)nb, 0);
        out.blocks.rows.assign((size_t)nb, 0);
        out.blocks.cols.assign((size_t)nb, 0);
        out.blocks.off.assign((size_t)nb, 0);
        check(qcm_plan_out_layout(plan.get(), &aux, &nb, out.blk_ptr.data(), out.blocks.q.data(),
                                  out.blocks.rows.data(), out.blocks.cols.data(), out.blocks.off.data()),
              "qcm_plan_out_layout");
        out.data = DeviceArray(out.elems());
        check(qcm_boundary_step(ctx_, plan.get(), ket.data.get(), b.data.get(), b.elems(), out.data.get(),
                                QCM_PREC_FP64),
              "qcm_boundary_step");
        return out;
    }

    qcm_ctx* ctx_ = nullptr;
    cudaStream_t stream_ = nullptr;
    bool herm_ = true;
};

// SiteProblem: the effective Hamiltonian of one (two-)site problem.
struct SiteProblem {
    const Boundary& left;
    const Boundary& right;
    const qcm_mpo_t& mpo;
};

// solve_ietl_jcd(SiteProblem&, init, parameters, ortho): the lowest eigenpair by
// Jacobi-Davidson (stopping rule |r| <= tol |theta|, at most maxiter steps), the
// solution kept orthogonal to the ortho vectors (same layout as init).
inline std::pair<double, MPSTensor> solve_ietl_jcd(Engine& engine, const SiteProblem& sp, const MPSTensor& init,
                                                   double tol, int maxiter,
                                                   const std::vector<const MPSTensor*>& ortho = {},
                                                   int precision = QCM_PREC_FP64, int* iterations = nullptr) {
    Plan p = engine.sigma_plan(init, sp.left, sp.right, sp.mpo);
    MPSTensor out = detail::like(init);
    std::vector<const double*> op;
    for (const MPSTensor* o : ortho) {
        if (o->elems() != init.elems()) throw error(QCM_E_INVALID, "solve_ietl_jcd: ortho vector of another layout");
        op.push_back(o->data.get());
    }
    double energy = 0.0;
    int32_t it = 0;
    check(qcm_jcd_solve(engine.ctx(), p.get(), sp.left.data.get(), sp.left.elems(), sp.right.data.get(),
                        sp.right.elems(), precision, init.data.get(), init.elems(), tol, maxiter,
                        op.empty() ? nullptr : op.data(), (int32_t)op.size(), out.data.get(), &energy, &it),
          "qcm_jcd_solve");
    if (iterations) *iterations = it;
    return {energy, std::move(out)};
}

// TwoSiteTensor of sites (i, i+1): the reduced two-site tensor (make_mps) and
// its split back into two site tensors with SVD truncation.
class TwoSiteTensor {
public:
    TwoSiteTensor(Engine& engine, const MPSTensor& A, const MPSTensor& B, int symmetry = QCM_SYM_SU2U1)
        : engine_(engine), sym_(symmetry), phys1_(A.phys), phys2_(B.phys), left_(A.left), right_(B.right) {
        const qcm_index_t p1 = A.phys.view(), al = A.left.view(), ar = A.right.view();
        const qcm_index_t p2 = B.phys.view(), bl = B.left.view(), br = B.right.view();
        const qcm_blocks_t ab = A.blocks.view(), bb = B.blocks.view();
        qcm_plan* raw = nullptr;
        check(qcm_plan_two_site(&p1, &al, &ar, &ab, &p2, &bl, &br, &bb, sym_, &raw), "qcm_plan_two_site");
        Plan plan(raw);
        detail::read_tensor_layout(
            [&](int32_t* nb, int32_t* q, int64_t* r, int64_t* c, int64_t* o, int32_t* n3, int32_t* iq, int64_t* is) {
                return qcm_plan_out_tensor(plan.get(), 0, nb, q, r, c, o, n3, iq, is);
            },
            theta_);
        theta_.data = DeviceArray(theta_.elems());
        check(qcm_ctx_run(engine_.ctx(), plan.get(), A.data.get(), B.data.get(), 0, nullptr, 0, theta_.data.get(),
                          QCM_PREC_FP64),
              "TwoSiteTensor");
    }

    // make_mps(): the reduced two-site tensor, left-paired
    const MPSTensor& make_mps() const { return theta_; }

    // tst << u: the optimised two-site tensor (same layout) replaces the data
    TwoSiteTensor& operator<<(const MPSTensor& u) {
        if (u.elems() != theta_.elems()) throw error(QCM_E_INVALID, "TwoSiteTensor <<: tensor of another layout");
        theta_.data = DeviceArray::copy_of(u.data.get(), u.elems(), engine_.stream());
        return *this;
    }

    // split_mps_l2r(Mmax, cutoff): A = U (left-normalised), B = S V^T
    std::tuple<MPSTensor, MPSTensor, qcm_trunc_t> split_mps_l2r(int64_t Mmax, double cutoff) {
        return split(true, Mmax, cutoff);
    }
    // split_mps_r2l(Mmax, cutoff): A = U S, B = V^T (right-normalised)
    std::tuple<MPSTensor, MPSTensor, qcm_trunc_t> split_mps_r2l(int64_t Mmax, double cutoff) {
        return split(false, Mmax, cutoff);
    }

private:
    std::tuple<MPSTensor, MPSTensor, qcm_trunc_t> split(bool l2r, int64_t Mmax, double cutoff) {
        const qcm_index_t p1 = phys1_.view(), p2 = phys2_.view(), l = left_.view(), r = right_.view();
        const qcm_blocks_t ub = theta_.blocks.view();
        qcm_trunc_t tr{};
        qcm_split_result* res = nullptr;
        check(qcm_split(engine_.ctx(), &p1, &p2, &l, &r, &ub, theta_.data.get(), l2r ? 1 : 0, Mmax, cutoff, sym_, &tr,
                        &res),
              "qcm_split");
        MPSTensor out[2];
        try {
            for (int w = 0; w < 2; ++w) {
                const double* d = nullptr;
                detail::read_tensor_layout(
                    [&](int32_t* nb, int32_t* q, int64_t* rr, int64_t* c, int64_t* o, int32_t* n3, int32_t* iq,
                        int64_t* is) { return qcm_split_result_tensor(res, w, nb, q, rr, c, o, n3, iq, is, &d); },
                    out[w]);
                out[w].data = DeviceArray::copy_of(d, out[w].elems(), engine_.stream());
            }
            // the copies read the result's memory: finish them before it is released
            cuda_check(cudaStreamSynchronize(engine_.stream()), "cudaStreamSynchronize");
        } catch (...) {
            qcm_split_result_destroy(res);
            throw;
        }
        qcm_split_result_destroy(res);
        return {std::move(out[0]), std::move(out[1]), tr};
    }

    Engine& engine_;
    int sym_;
    IndexArr phys1_, phys2_, left_, right_;
    MPSTensor theta_;
};

}  // namespace qcm
