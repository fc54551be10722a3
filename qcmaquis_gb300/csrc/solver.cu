// The execution context and the Jacobi-Davidson eigensolver of the two-site
// problem, in native code.
//
// qcm_ctx owns everything a sequence of plan runs needs besides the caller's
// tensors: one CUDA stream, the plans' scratch slots and operand-image buffer,
// FP32 shadows of the boundaries for the mixed-precision forms, and the
// eigensolver's basis vectors and reduction partials.  Its buffers only grow;
// calls on one context run in order on its stream and are not reentrant.
//
// qcm_jcd_solve restates solve_ietl_jcd (dmrg/framework/dmrg/optimize/
// ietl_jacobi_davidson.h:16-77) over jacobi_davidson::calculate_eigenvalue
// (dmrg/framework/ietl/jacobi.h:361-451) with zero GMRES steps, the live path's
// setting (jcd_gmres_solver with max_iter 0, jacobi.h:99-138):
//   modified Gram-Schmidt with one refinement pass when the norm fell below
//   kappa = 0.25 of its start (jacobi.h:385-390), the orthogonality constraints
//   of excited states (ietl_jacobi_davidson.h:28-49, SingleSiteVS::project),
//   normalisation, sigma, the new column of the projected matrix, its smallest
//   eigenpair (dsyevx in the reference; a cyclic Jacobi here), u = V s,
//   uA = VA s, r = uA - theta u, stop when |r| <= tol |theta|, |r| < tol or
//   after maxiter steps, else t = -r + (r.u / u.u) u.
// Every coefficient of the Gram-Schmidt passes, projections and the correction
// stays on the device (a kernel reads it where the next kernel needs it), so an
// iteration synchronises the host twice: for the projected matrix column and for
// the residual norm.  Reductions are two-pass with a fixed combine order, so a
// solve is bitwise repeatable.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "plan.hpp"

namespace qcm {
namespace {

#define SOL_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t err__ = (call);                                                     \
        if (err__ != cudaSuccess) {                                                     \
            set_error(std::string(#call) + ": " + cudaGetErrorString(err__));           \
            return QCM_E_CUDA;                                                          \
        }                                                                               \
    } while (0)

constexpr int SR_THREADS = 256;
constexpr int SR_BLOCKS = 304;     // 2 x 152 SMs
constexpr int SR_MAXVEC = 64;      // vectors one multi-dot handles
constexpr int NSCAL = 64;          // device scalar slots of a context

__device__ __forceinline__ double wsum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double bsum(double v) {
    __shared__ double ws[SR_THREADS / 32];
    v = wsum(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) ws[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = lane < SR_THREADS / 32 ? ws[lane] : 0.0;
        r = wsum(r);
    }
    return r;   // thread 0
}

struct VecList { const double* x[SR_MAXVEC]; };

// partial[k * gridDim.x + block] = block's share of <x_k, y>
__global__ void __launch_bounds__(SR_THREADS)
sr_partial(VecList v, int nvec, const double* __restrict__ y, int64_t n, double* __restrict__ partial) {
    for (int k = 0; k < nvec; ++k) {
        const double* __restrict__ x = v.x[k];
        double s = 0.0;
        for (int64_t i = (int64_t)blockIdx.x * SR_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * SR_THREADS)
            s = fma(x[i], y[i], s);
        s = bsum(s);
        if (threadIdx.x == 0) partial[(int64_t)k * gridDim.x + blockIdx.x] = s;
    }
}

// out[k] = sum of the partials (sqrt with do_sqrt)
__global__ void __launch_bounds__(SR_THREADS)
sr_final(const double* __restrict__ partial, int nparts, int nvec, double* __restrict__ out, int do_sqrt) {
    for (int k = 0; k < nvec; ++k) {
        double s = 0.0;
        for (int i = threadIdx.x; i < nparts; i += SR_THREADS) s += partial[(int64_t)k * nparts + i];
        s = bsum(s);
        if (threadIdx.x == 0) out[k] = do_sqrt ? sqrt(s) : s;
    }
}

// y += scale * c * x with c = num[0] (den == null) or num[0] / den[0]; skipped
// unless gate_a == null or gate_a[0] < kappa * gate_b[0]
__global__ void sr_axpy_dev(const double* __restrict__ x, double* __restrict__ y, int64_t n,
                            const double* __restrict__ num, const double* __restrict__ den, double scale,
                            const double* __restrict__ gate_a, const double* __restrict__ gate_b, double kappa) {
    if (gate_a && !(gate_a[0] < kappa * gate_b[0])) return;
    const double c = scale * (den ? num[0] / den[0] : num[0]);
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = fma(c, x[i], y[i]);
}

// x *= 1 / nrm[0]
__global__ void sr_scale_inv(double* __restrict__ x, int64_t n, const double* __restrict__ nrm) {
    const double c = 1.0 / nrm[0];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        x[i] *= c;
}

// t = -r + (ru[0] / uu[0]) u
__global__ void sr_correction(double* __restrict__ t, const double* __restrict__ r, const double* __restrict__ u,
                              int64_t n, const double* __restrict__ ru, const double* __restrict__ uu) {
    const double c = ru[0] / uu[0];
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        t[i] = fma(c, u[i], -r[i]);
}

// y = a x + b y
__global__ void sr_axpby(double a, const double* __restrict__ x, double b, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = b == 0.0 ? a * x[i] : fma(a, x[i], b * y[i]);
}

struct LinList { const double* x[SR_MAXVEC]; double c[SR_MAXVEC]; };

__global__ void sr_lincomb(LinList a, int nvec, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < nvec; ++k) s = fma(a.c[k], a.x[k][i], s);
        y[i] = s;
    }
}

__global__ void sr_to_f32(const double* __restrict__ x, float* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (float)x[i];
}

inline unsigned grid_for(int64_t n) { return (unsigned)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, 152 * 8)); }

// Eigenpairs of a small symmetric matrix (row-major k x k) by cyclic Jacobi
// rotations; eigenvalues ascending, eigenvectors as the columns of Z.
void small_sym_eig(int k, std::vector<double> A, std::vector<double>& w, std::vector<double>& Z) {
    Z.assign((size_t)k * k, 0.0);
    for (int i = 0; i < k; ++i) Z[(size_t)i * k + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, dia = 0.0;
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j) (i == j ? dia : off) += A[(size_t)i * k + j] * A[(size_t)i * k + j];
        if (off <= 1e-32 * dia || off == 0.0) break;
        for (int p = 0; p < k; ++p)
            for (int q = p + 1; q < k; ++q) {
                const double apq = A[(size_t)p * k + q];
                if (apq == 0.0) continue;
                const double app = A[(size_t)p * k + p], aqq = A[(size_t)q * k + q];
                const double tau = (aqq - app) / (2.0 * apq);
                const double t = std::copysign(1.0, tau) / (std::fabs(tau) + std::hypot(1.0, tau));
                const double c = 1.0 / std::sqrt(1.0 + t * t), s = t * c;
                for (int r = 0; r < k; ++r) {   // A <- A J (columns p, q)
                    const double x = A[(size_t)r * k + p], y = A[(size_t)r * k + q];
                    A[(size_t)r * k + p] = c * x - s * y;
                    A[(size_t)r * k + q] = s * x + c * y;
                }
                for (int r = 0; r < k; ++r) {   // A <- J^T A (rows p, q)
                    const double x = A[(size_t)p * k + r], y = A[(size_t)q * k + r];
                    A[(size_t)p * k + r] = c * x - s * y;
                    A[(size_t)q * k + r] = s * x + c * y;
                }
                for (int r = 0; r < k; ++r) {
                    const double x = Z[(size_t)r * k + p], y = Z[(size_t)r * k + q];
                    Z[(size_t)r * k + p] = c * x - s * y;
                    Z[(size_t)r * k + q] = s * x + c * y;
                }
            }
    }
    std::vector<int> ord(k);
    for (int i = 0; i < k; ++i) ord[i] = i;
    std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return A[(size_t)a * k + a] < A[(size_t)b * k + b]; });
    w.resize(k);
    std::vector<double> Zs((size_t)k * k);
    for (int c = 0; c < k; ++c) {
        w[c] = A[(size_t)ord[c] * k + ord[c]];
        for (int r = 0; r < k; ++r) Zs[(size_t)r * k + c] = Z[(size_t)r * k + ord[c]];
    }
    Z.swap(Zs);
}

}  // namespace
}  // namespace qcm

using namespace qcm;

struct qcm_ctx {
    int device = -1;
    cudaStream_t stream = nullptr;
    void* scratch[3] = {nullptr, nullptr, nullptr};
    size_t scratch_bytes[3] = {0, 0, 0};
    void* img = nullptr;
    size_t img_bytes = 0;
    float* shadow[2] = {nullptr, nullptr};
    size_t shadow_elems[2] = {0, 0};
    double* vecs = nullptr;
    size_t vec_elems = 0;
    double* partial = nullptr;
    double* scal = nullptr;     // device scalars
    double* h_buf = nullptr;    // pinned host copy area (NSCAL + SR_MAXVEC doubles)
};

struct qcm_split_result {
    double* a = nullptr;
    double* b = nullptr;
    std::vector<Blk> layout_a, layout_b;
    Idx idx_a[3], idx_b[3];
};

namespace {

int grow(void** p, size_t* cap, size_t bytes) {
    if (bytes <= *cap && *p) return QCM_OK;
    if (*p) SOL_CUDA(cudaFree(*p));
    *p = nullptr;
    *cap = 0;
    if (cudaMalloc(p, std::max<size_t>(bytes, 256)) != cudaSuccess) {
        *p = nullptr;
        set_error("qcm_ctx: device allocation of " + std::to_string(bytes) + " bytes failed");
        return QCM_E_NOMEM;
    }
    *cap = std::max<size_t>(bytes, 256);
    return QCM_OK;
}

int check_ctx(qcm_ctx* c) {
    if (!c) { set_error("null context"); return QCM_E_INVALID; }
    int dev = 0;
    SOL_CUDA(cudaGetDevice(&dev));
    if (dev != c->device) { set_error("the context belongs to another device"); return QCM_E_STATE; }
    return QCM_OK;
}

// <x_k, y> for k < nvec into the device array out (sqrt with nrm)
int dots(qcm_ctx* c, const double* const* x, int nvec, const double* y, int64_t n, double* out, bool nrm = false) {
    VecList v;
    for (int k = 0; k < SR_MAXVEC; ++k) v.x[k] = k < nvec ? x[k] : nullptr;
    sr_partial<<<SR_BLOCKS, SR_THREADS, 0, c->stream>>>(v, nvec, y, n, c->partial);
    sr_final<<<1, SR_THREADS, 0, c->stream>>>(c->partial, SR_BLOCKS, nvec, out, nrm ? 1 : 0);
    SOL_CUDA(cudaGetLastError());
    return QCM_OK;
}

int fetch(qcm_ctx* c, const double* dev, int n, double* host) {
    SOL_CUDA(cudaMemcpyAsync(c->h_buf, dev, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    SOL_CUDA(cudaStreamSynchronize(c->stream));
    std::memcpy(host, c->h_buf, sizeof(double) * n);
    return QCM_OK;
}

// bufs for a plan run on the context: scratch and images from the context; FP32
// shadows of the boundaries for the mixed forms
int prepare_run(qcm_ctx* c, qcm_plan* plan, int32_t precision, const double* left, int64_t left_elems,
                const double* right, int64_t right_elems, bool convert, double* bufs[QCM_NBUF], uint32_t* mask) {
    int rc = qcm_plan_upload(plan);
    if (rc) return rc;
    int64_t out = 0, sc[3] = {0, 0, 0};
    if ((rc = qcm_plan_sizes(plan, &out, sc))) return rc;
    for (int i = 0; i < 3; ++i)
        if ((rc = grow(&c->scratch[i], &c->scratch_bytes[i], sizeof(double) * (size_t)std::max<int64_t>(sc[i], 1))))
            return rc;
    const bool img_form = precision == QCM_PREC_BF16X3 || precision == QCM_PREC_BF16X2;
    int64_t ib = 0;
    if (img_form) {
        if ((rc = qcm_plan_image_bytes(plan, &ib))) return rc;
        if ((rc = grow(&c->img, &c->img_bytes, (size_t)std::max<int64_t>(ib, 1)))) return rc;
    }
    for (int i = 0; i < QCM_NBUF; ++i) bufs[i] = nullptr;
    bufs[QCM_BUF_LEFT] = const_cast<double*>(left);
    bufs[QCM_BUF_RIGHT] = const_cast<double*>(right);
    bufs[QCM_BUF_S0] = (double*)c->scratch[0];
    bufs[QCM_BUF_S1] = (double*)c->scratch[1];
    bufs[QCM_BUF_S2] = (double*)c->scratch[2];
    bufs[QCM_BUF_IMG] = img_form && ib > 0 ? (double*)c->img : nullptr;
    *mask = 0;
    if (precision != QCM_PREC_FP64) {
        *mask = (1u << QCM_BUF_S0) | (1u << QCM_BUF_S1) | (1u << QCM_BUF_S2);
        const double* src[2] = {left, right};
        const int64_t len[2] = {left_elems, right_elems};
        const int slot[2] = {QCM_BUF_LEFT, QCM_BUF_RIGHT};
        for (int s = 0; s < 2; ++s) {
            if (!src[s]) continue;
            if (len[s] <= 0) { set_error("mixed precision needs the boundary lengths"); return QCM_E_INVALID; }
            size_t cap = c->shadow_elems[s] * sizeof(float);
            if ((rc = grow((void**)&c->shadow[s], &cap, sizeof(float) * (size_t)len[s]))) return rc;
            c->shadow_elems[s] = cap / sizeof(float);
            if (convert) {
                sr_to_f32<<<grid_for(len[s]), 256, 0, c->stream>>>(src[s], c->shadow[s], len[s]);
                SOL_CUDA(cudaGetLastError());
            }
            bufs[slot[s]] = (double*)c->shadow[s];
            *mask |= 1u << slot[s];
        }
    }
    return QCM_OK;
}

}  // namespace

extern "C" {

int qcm_ctx_create(void* stream, qcm_ctx** out) {
    if (!out) { set_error("qcm_ctx_create: null output"); return QCM_E_INVALID; }
    *out = nullptr;
    auto* c = new qcm_ctx();
    if (cudaGetDevice(&c->device) != cudaSuccess) { delete c; set_error("qcm_ctx_create: no device"); return QCM_E_CUDA; }
    c->stream = (cudaStream_t)stream;
    if (cudaMalloc(&c->partial, sizeof(double) * SR_BLOCKS * SR_MAXVEC) != cudaSuccess ||
        cudaMalloc(&c->scal, sizeof(double) * NSCAL) != cudaSuccess ||
        cudaMallocHost(&c->h_buf, sizeof(double) * (NSCAL + SR_MAXVEC)) != cudaSuccess) {
        qcm_ctx_destroy(c);
        set_error("qcm_ctx_create: allocation failed");
        return QCM_E_NOMEM;
    }
    *out = c;
    return QCM_OK;
}

int qcm_ctx_set_stream(qcm_ctx* c, void* stream) {
    int rc = check_ctx(c);
    if (rc) return rc;
    c->stream = (cudaStream_t)stream;
    return QCM_OK;
}

void qcm_ctx_destroy(qcm_ctx* c) {
    if (!c) return;
    for (auto* p : c->scratch) cudaFree(p);
    cudaFree(c->img);
    cudaFree(c->shadow[0]);
    cudaFree(c->shadow[1]);
    cudaFree(c->vecs);
    cudaFree(c->partial);
    cudaFree(c->scal);
    if (c->h_buf) cudaFreeHost(c->h_buf);
    delete c;
}

int qcm_ctx_run(qcm_ctx* c, qcm_plan* plan, const double* ket, const double* left, int64_t left_elems,
                const double* right, int64_t right_elems, double* out, int32_t precision) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!plan) { set_error("qcm_ctx_run: null plan"); return QCM_E_INVALID; }
    double* bufs[QCM_NBUF];
    uint32_t mask = 0;
    if ((rc = prepare_run(c, plan, precision, left, left_elems, right, right_elems, true, bufs, &mask))) return rc;
    bufs[QCM_BUF_KET] = const_cast<double*>(ket);
    bufs[QCM_BUF_OUT] = out;
    return qcm_plan_run_typed(plan, bufs, mask, precision, c->stream, 0, -1);
}

int qcm_boundary_step(qcm_ctx* c, qcm_plan* plan, const double* mps, const double* boundary, int64_t boundary_elems,
                      double* out, int32_t precision) {
    if (!plan || (plan->kind != PK_BLEFT && plan->kind != PK_BRIGHT)) {
        set_error("qcm_boundary_step: not a boundary-step plan");
        return QCM_E_STATE;
    }
    const bool left = plan->kind == PK_BLEFT;
    return qcm_ctx_run(c, plan, mps, left ? boundary : nullptr, left ? boundary_elems : 0, left ? nullptr : boundary,
                       left ? 0 : boundary_elems, out, precision);
}

int qcm_split(qcm_ctx* c, const qcm_index_t* phys1, const qcm_index_t* phys2, const qcm_index_t* left_i,
              const qcm_index_t* right_i, const qcm_blocks_t* u, const double* u_dev, int32_t l2r, int64_t Mmax,
              double cutoff, int32_t symmetry, qcm_trunc_t* trunc, qcm_split_result** out) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!u_dev || !trunc || !out) { set_error("qcm_split: null argument"); return QCM_E_INVALID; }
    if (symmetry != QCM_SYM_SU2U1 && symmetry != QCM_SYM_TWOU1 && symmetry != QCM_SYM_U1) {
        set_error("qcm_split: unknown symmetry");
        return QCM_E_INVALID;
    }
    *out = nullptr;
    qcm_plan* sp = nullptr;
    qcm_svd* svd = nullptr;
    qcm_plan* ap = nullptr;
    double *theta = nullptr, *work = nullptr, *U = nullptr, *S = nullptr, *Vt = nullptr;
    auto* res = new qcm_split_result();
    auto cleanup = [&](int code) {
        if (sp) qcm_plan_destroy(sp);
        if (ap) qcm_plan_destroy(ap);
        if (svd) qcm_svd_destroy(svd);
        cudaFree(theta); cudaFree(work); cudaFree(U); cudaFree(S); cudaFree(Vt);
        if (code) qcm_split_result_destroy(res);
        return code;
    };
    try {
        sp = build_split(read_index(phys1), read_index(phys2), read_index(left_i), read_index(right_i),
                         read_blocks(u), symmetry != QCM_SYM_SU2U1);
    } catch (const std::exception& e) {
        set_error(std::string("qcm_split: ") + e.what());
        return cleanup(QCM_E_INVALID);
    }
    // the both-paired matrix
    if (cudaMalloc(&theta, sizeof(double) * std::max<int64_t>(sp->out_elems, 1)) != cudaSuccess) {
        set_error("qcm_split: allocation failed");
        return cleanup(QCM_E_NOMEM);
    }
    if ((rc = qcm_ctx_run(c, sp, u_dev, nullptr, 0, nullptr, 0, theta, QCM_PREC_FP64))) return cleanup(rc);
    // batched SVD of its blocks and the cut
    const size_t nb = sp->out_bm.size();
    std::vector<int64_t> rows(nb), cols(nb), offs(nb);
    for (size_t k = 0; k < nb; ++k) {
        rows[k] = sp->out_bm[k].rows;
        cols[k] = sp->out_bm[k].cols;
        offs[k] = sp->out_bm[k].off;
    }
    if ((rc = qcm_svd_create((int32_t)nb, rows.data(), cols.data(), offs.data(), &svd))) return cleanup(rc);
    int64_t we = 0, ue = 0, se = 0, ve = 0;
    qcm_svd_sizes(svd, &we, &ue, &se, &ve);
    if (cudaMalloc(&work, sizeof(double) * std::max<int64_t>(we, 1)) != cudaSuccess ||
        cudaMalloc(&U, sizeof(double) * std::max<int64_t>(ue, 1)) != cudaSuccess ||
        cudaMalloc(&S, sizeof(double) * std::max<int64_t>(se, 1)) != cudaSuccess ||
        cudaMalloc(&Vt, sizeof(double) * std::max<int64_t>(ve, 1)) != cudaSuccess) {
        set_error("qcm_split: allocation failed");
        return cleanup(QCM_E_NOMEM);
    }
    if ((rc = qcm_svd_run(svd, theta, work, U, S, Vt, c->stream))) return cleanup(rc);
    std::vector<int64_t> s_off(nb), u_off(nb), vt_off(nb), blk(nb + 1, 0), keep(std::max<size_t>(nb, 1));
    qcm_svd_block_offsets(svd, s_off.data(), u_off.data(), vt_off.data());
    for (size_t k = 0; k < nb; ++k) blk[k + 1] = blk[k] + std::min(rows[k], cols[k]);
    if ((rc = qcm_truncation_cut(S, (int32_t)nb, blk.data(), Mmax, cutoff, 0, keep.data(), trunc, c->stream)))
        return cleanup(rc);
    std::vector<double> Sh(std::max<int64_t>(se, 1));
    if (se > 0) {
        SOL_CUDA(cudaMemcpyAsync(Sh.data(), S, sizeof(double) * se, cudaMemcpyDeviceToHost, c->stream));
        SOL_CUDA(cudaStreamSynchronize(c->stream));
    }
    try {
        BM both;
        both.b = sp->out_bm;
        std::vector<int64_t> kdim(nb);
        for (size_t k = 0; k < nb; ++k) kdim[k] = std::min(rows[k], cols[k]);
        ap = build_assemble(sp->out_phys, sp->out2_phys, sp->out_left, sp->out_right, both, u_off.data(),
                            vt_off.data(), kdim.data(), keep.data(), Sh.data(), s_off.data(), l2r != 0);
    } catch (const std::exception& e) {
        set_error(std::string("qcm_split: ") + e.what());
        return cleanup(QCM_E_INVALID);
    }
    // the two site tensors, owned by the result
    if (cudaMalloc(&res->a, sizeof(double) * std::max<int64_t>(ap->out_elems, 1)) != cudaSuccess ||
        cudaMalloc(&res->b, sizeof(double) * std::max<int64_t>(ap->scratch[2], 1)) != cudaSuccess) {
        set_error("qcm_split: allocation failed");
        return cleanup(QCM_E_NOMEM);
    }
    if ((rc = qcm_plan_upload(ap))) return cleanup(rc);
    {
        int64_t oe = 0, sc[3] = {0, 0, 0};
        qcm_plan_sizes(ap, &oe, sc);
        if ((rc = grow(&c->scratch[0], &c->scratch_bytes[0], sizeof(double) * (size_t)std::max<int64_t>(sc[0], 1))))
            return cleanup(rc);
        double* bufs[QCM_NBUF] = {U, Vt, nullptr, res->a, (double*)c->scratch[0], nullptr, res->b, nullptr};
        if ((rc = qcm_plan_run_typed(ap, bufs, 0, QCM_PREC_FP64, c->stream, 0, -1))) return cleanup(rc);
    }
    SOL_CUDA(cudaStreamSynchronize(c->stream));
    res->layout_a = ap->out_bm;
    res->layout_b = ap->out2_bm;
    res->idx_a[0] = ap->out_phys; res->idx_a[1] = ap->out_left; res->idx_a[2] = ap->out_right;
    res->idx_b[0] = ap->out2_phys; res->idx_b[1] = ap->out2_left; res->idx_b[2] = ap->out2_right;
    *out = res;
    return cleanup(QCM_OK);
}

int qcm_split_result_tensor(const qcm_split_result* r, int32_t which, int32_t* nblocks, int32_t* q, int64_t* rows,
                            int64_t* cols, int64_t* off, int32_t* n_idx3, int32_t* idx_q, int64_t* idx_size,
                            const double** data) {
    if (!r || (which != 0 && which != 1)) { set_error("qcm_split_result_tensor: invalid arguments"); return QCM_E_INVALID; }
    const auto& bm = which == 0 ? r->layout_a : r->layout_b;
    const Idx* ix = which == 0 ? r->idx_a : r->idx_b;
    if (nblocks) *nblocks = (int32_t)bm.size();
    for (size_t k = 0; k < bm.size(); ++k) {
        if (q) { q[4 * k] = bm[k].lc.n; q[4 * k + 1] = bm[k].lc.s; q[4 * k + 2] = bm[k].rc.n; q[4 * k + 3] = bm[k].rc.s; }
        if (rows) rows[k] = bm[k].rows;
        if (cols) cols[k] = bm[k].cols;
        if (off) off[k] = bm[k].off;
    }
    int64_t base = 0;
    for (int i = 0; i < 3; ++i) {
        if (n_idx3) n_idx3[i] = (int32_t)ix[i].d.size();
        for (size_t k = 0; k < ix[i].d.size(); ++k) {
            if (idx_q) { idx_q[2 * (base + k)] = ix[i].d[k].first.n; idx_q[2 * (base + k) + 1] = ix[i].d[k].first.s; }
            if (idx_size) idx_size[base + k] = ix[i].d[k].second;
        }
        base += (int64_t)ix[i].d.size();
    }
    if (data) *data = which == 0 ? r->a : r->b;
    return QCM_OK;
}

void qcm_split_result_destroy(qcm_split_result* r) {
    if (!r) return;
    cudaFree(r->a);
    cudaFree(r->b);
    delete r;
}

int qcm_jcd_solve(qcm_ctx* c, qcm_plan* sigma, const double* left, int64_t left_elems, const double* right,
                  int64_t right_elems, int32_t precision, const double* init, int64_t n, double tol, int32_t maxiter,
                  const double* const* ortho, int32_t n_ortho, double* out_vec, double* out_energy,
                  int32_t* out_iters) {
    int rc = check_ctx(c);
    if (rc) return rc;
    if (!sigma || sigma->kind != PK_SIGMA) { set_error("qcm_jcd_solve: not a sigma plan"); return QCM_E_STATE; }
    if (!init || !out_vec || !out_energy || !out_iters || n <= 0) {
        set_error("qcm_jcd_solve: invalid arguments");
        return QCM_E_INVALID;
    }
    if (maxiter < 1 || maxiter > 32) { set_error("qcm_jcd_solve: maxiter must be in 1..32"); return QCM_E_RANGE; }
    if (n_ortho < 0 || n_ortho > 16 || (n_ortho > 0 && !ortho)) {
        set_error("qcm_jcd_solve: at most 16 orthogonality constraints");
        return QCM_E_RANGE;
    }
    if (sigma->out_elems != n) { set_error("qcm_jcd_solve: vector length differs from the plan's"); return QCM_E_INVALID; }
    // vectors: V[maxiter], VA[maxiter], u, uA, t, tmp, local ortho copies
    const int nv = 2 * maxiter + 4 + n_ortho;
    size_t cap = c->vec_elems * sizeof(double);
    if ((rc = grow((void**)&c->vecs, &cap, sizeof(double) * (size_t)n * nv))) return rc;
    c->vec_elems = cap / sizeof(double);
    double* V = c->vecs;
    double* VA = V + (size_t)maxiter * n;
    double* u = VA + (size_t)maxiter * n;
    double* uA = u + n;
    double* t = uA + n;
    double* tmp = t + n;
    double* loc = tmp + n;
    double* S = c->scal;   // scalar slots: 0 tau, 1 nu, 2 coef, 3 coef2, 4 nrm, 5.. multi-dot column
    const cudaStream_t st = c->stream;
    const unsigned g = grid_for(n);
    double* bufs[QCM_NBUF];
    uint32_t mask = 0;
    if ((rc = prepare_run(c, sigma, precision, left, left_elems, right, right_elems, true, bufs, &mask))) return rc;
    auto apply = [&](const double* x, double* y) -> int {
        double* b[QCM_NBUF];
        for (int i = 0; i < QCM_NBUF; ++i) b[i] = bufs[i];
        b[QCM_BUF_KET] = const_cast<double*>(x);
        b[QCM_BUF_OUT] = y;
        return qcm_plan_run_typed(sigma, b, mask, precision, st, 0, -1);
    };
    auto dot1 = [&](const double* x, const double* y, double* o) { return dots(c, &x, 1, y, n, o, false); };
    auto nrm = [&](const double* x, double* o) { return dots(c, &x, 1, x, n, o, true); };
    auto axpy_d = [&](const double* x, double* y, const double* num, const double* den, double scale,
                      const double* ga = nullptr, const double* gb = nullptr, double kap = 0.0) -> int {
        sr_axpy_dev<<<g, 256, 0, st>>>(x, y, n, num, den, scale, ga, gb, kap);
        SOL_CUDA(cudaGetLastError());
        return QCM_OK;
    };
    const double completeness = 1e-10;
    // orthonormalised constraints (ietl_jacobi_davidson.h:28-49)
    std::vector<double*> local;
    for (int32_t o = 0; o < n_ortho && o < n - 1; ++o) {
        double* v = loc + (size_t)o * n;
        SOL_CUDA(cudaMemcpyAsync(v, ortho[o], sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        for (double* q : local) {
            if ((rc = dot1(q, v, S + 2))) return rc;
            if ((rc = axpy_d(q, v, S + 2, nullptr, -1.0))) return rc;
        }
        double nv_h = 0.0;
        if ((rc = nrm(v, S + 4)) || (rc = fetch(c, S + 4, 1, &nv_h))) return rc;
        if (nv_h > completeness) {
            sr_scale_inv<<<g, 256, 0, st>>>(v, n, S + 4);
            SOL_CUDA(cudaGetLastError());
            local.push_back(v);
        }
    }
    auto project = [&](double* x) -> int {
        for (double* q : local) {
            int r2;
            if ((r2 = dot1(q, x, S + 2)) || (r2 = dot1(q, q, S + 3)) || (r2 = axpy_d(q, x, S + 2, S + 3, -1.0)))
                return r2;
        }
        return QCM_OK;
    };
    if (!local.empty()) {
        SOL_CUDA(cudaMemcpyAsync(tmp, init, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        for (double* q : local) {
            if ((rc = dot1(tmp, q, S + 2)) || (rc = axpy_d(q, tmp, S + 2, nullptr, -1.0))) return rc;
        }
        double nt_h = 0.0;
        if ((rc = nrm(tmp, S + 4)) || (rc = fetch(c, S + 4, 1, &nt_h))) return rc;
        if (nt_h < completeness) {
            // nothing of the start vector is left: no solve (<init|A init>, init, 0)
            if ((rc = apply(init, uA))) return rc;
            double e = 0.0;
            if ((rc = dot1(init, uA, S + 2)) || (rc = fetch(c, S + 2, 1, &e))) return rc;
            SOL_CUDA(cudaMemcpyAsync(out_vec, init, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
            SOL_CUDA(cudaStreamSynchronize(st));
            *out_energy = e;
            *out_iters = 0;
            return QCM_OK;
        }
    }
    const double kappa = 0.25;
    std::vector<double> M((size_t)maxiter * maxiter, 0.0), col(maxiter), w, Z;
    SOL_CUDA(cudaMemcpyAsync(t, init, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    if ((rc = project(t))) return rc;
    int it = 0;
    double theta = 0.0;
    while (true) {
        double* Vi = V + (size_t)it * n;
        // modified Gram-Schmidt, one refinement pass when |t| dropped below kappa |t_start|
        if ((rc = nrm(t, S + 0))) return rc;
        for (int i = 0; i < it; ++i)
            if ((rc = dot1(V + (size_t)i * n, t, S + 2)) || (rc = axpy_d(V + (size_t)i * n, t, S + 2, nullptr, -1.0)))
                return rc;
        if ((rc = nrm(t, S + 1))) return rc;
        for (int i = 0; i < it; ++i)
            if ((rc = dot1(V + (size_t)i * n, t, S + 2)) ||
                (rc = axpy_d(V + (size_t)i * n, t, S + 2, nullptr, -1.0, S + 1, S + 0, kappa)))
                return rc;
        if ((rc = project(t))) return rc;
        if ((rc = nrm(t, S + 4))) return rc;
        sr_scale_inv<<<g, 256, 0, st>>>(t, n, S + 4);
        SOL_CUDA(cudaGetLastError());
        SOL_CUDA(cudaMemcpyAsync(Vi, t, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
        // sigma and the new column of the projected matrix
        if ((rc = apply(Vi, VA + (size_t)it * n))) return rc;
        std::vector<const double*> vs(it + 1);
        for (int i = 0; i <= it; ++i) vs[i] = V + (size_t)i * n;
        if ((rc = dots(c, vs.data(), it + 1, VA + (size_t)it * n, n, S + 5))) return rc;
        if ((rc = fetch(c, S + 5, it + 1, col.data()))) return rc;
        for (int i = 0; i <= it; ++i) M[(size_t)i * maxiter + it] = col[i];
        const int k = it + 1;
        std::vector<double> Ms((size_t)k * k);
        for (int i = 0; i < k; ++i)
            for (int j = 0; j < k; ++j)
                Ms[(size_t)i * k + j] = i <= j ? M[(size_t)i * maxiter + j] : M[(size_t)j * maxiter + i];
        small_sym_eig(k, Ms, w, Z);
        theta = w[0];
        LinList lu, la;
        for (int i = 0; i < SR_MAXVEC; ++i) {
            lu.x[i] = i < k ? V + (size_t)i * n : nullptr;
            la.x[i] = i < k ? VA + (size_t)i * n : nullptr;
            lu.c[i] = la.c[i] = i < k ? Z[(size_t)i * k + 0] : 0.0;
        }
        sr_lincomb<<<g, 256, 0, st>>>(lu, k, u, n);
        sr_lincomb<<<g, 256, 0, st>>>(la, k, uA, n);
        SOL_CUDA(cudaGetLastError());
        if ((rc = project(uA))) return rc;
        sr_axpby<<<g, 256, 0, st>>>(-theta, u, 1.0, uA, n);   // r = uA - theta u (in uA)
        SOL_CUDA(cudaGetLastError());
        ++it;
        double rn = 0.0;
        if ((rc = nrm(uA, S + 4)) || (rc = fetch(c, S + 4, 1, &rn))) return rc;
        if (rn <= tol * std::fabs(theta) || rn < tol || it >= maxiter) break;
        if ((rc = dot1(uA, u, S + 2)) || (rc = dot1(u, u, S + 3))) return rc;
        sr_correction<<<g, 256, 0, st>>>(t, uA, u, n, S + 2, S + 3);
        SOL_CUDA(cudaGetLastError());
    }
    SOL_CUDA(cudaMemcpyAsync(out_vec, u, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    SOL_CUDA(cudaStreamSynchronize(st));
    *out_energy = theta;
    *out_iters = it;
    return QCM_OK;
}

}  // extern "C"
