// Dense FP64 factorisations of the truncation and canonicalisation steps, on the
// GPU, for a batch of independent blocks at once.
//
// The reference factorises each block of a block matrix separately on the host
// with LAPACK (alps gesvd / heevd, dmrg/alps/src/alps/numeric/matrix/
// algorithms.hpp:248-261, 402-421; called per block from svd_truncate /
// heev_truncate, bm/block_matrix_algorithms.h:163-333, 387-440, and qr / lq,
// :442-492).  Here every block of a batch is factorised by one-sided (Hestenes)
// Jacobi in FP64 (Demmel-Veselic, "Jacobi's method is more accurate than QR",
// SIAM J. Matrix Anal. Appl. 13 (1992)):
//
//   * the working matrix W (p x q, p >= q: the block, or its transpose when it
//     has fewer rows than columns) has its columns pairwise orthogonalised by
//     plane rotations, which are accumulated into V (q x q, starting at I);
//   * the columns are cut into panels of bw columns (bw = 16 or 8 by default: the
//     widest whose two panels of W and V fit in shared memory; 4 or 2 on request)
//     and one kernel
//     launch is one round of a round-robin tournament over the panel pairs of
//     every block (nb' - 1 rounds per sweep, nb' = the panel count rounded up to
//     even).  The CTA of a panel pair loads its 2 bw columns of W and of V into
//     shared memory and rotates there the column pairs across the two panels
//     (and, in a sweep's first round, those inside each panel) -- the same
//     rotations, from fresh inner products of the current columns -- then writes
//     the columns back.  Every column pair is rotated once per sweep, the work
//     of the single-column rounds in 1/bw of their launches and traffic.  A
//     batch whose widest block is too tall for two panels of 8 columns uses
//     single column pairs, one warp per pair and one round per launch
//     (q' - 1 rounds per sweep, q' = q rounded up to even).  GB300's FP64 rate
//     bounds both forms: the panels save launches (a tenth) rather than time;
//   * a block stops after a sweep that rotated no pair (|w_i.w_j| <= tol *
//     |w_i| |w_j| for all pairs, tol = sqrt(p) eps as in LAPACK's dgesvj);
//     blocks with fewer columns run more sweeps in the same launches;
//   * the singular values are the column norms; they are sorted descending per
//     block and U, S, Vt are written in the layout of gesvd('S','S').
//
// For a symmetric positive semi-definite block (a density matrix) the same
// factorisation is its eigendecomposition (U = eigenvectors, S = eigenvalues,
// descending, as heev_truncate orders them).
//
// The truncation cut (estimate_truncation, block_matrix_algorithms.h:211-333)
// runs on the device too: one CTA sorts all singular values (or eigenvalues)
// of the batch, takes evalscut = max(cutoff * s0, s[Mmax]), keeps every value
// >= evalscut (Mmax + 1 values when there is no tie, as the reference does),
// and sums the discarded weight in a fixed order.
//
// Every wait is a kernel boundary; there are no spin-waits.  A block that has
// not converged after QCM_SVD_MAX_SWEEPS sweeps is finished as it is and
// flagged (qcm_svd_run returns QCM_E_RANGE with its index).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "plan.hpp"

namespace qcm {

#define FCT_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t err__ = (call);                                                     \
        if (err__ != cudaSuccess) {                                                     \
            set_error(std::string(#call) + ": " + cudaGetErrorString(err__));           \
            return QCM_E_CUDA;                                                          \
        }                                                                               \
    } while (0)

constexpr int SVD_MAX_SWEEPS = 40;
// rotation threshold |w_i.w_j| <= tol |w_i| |w_j| with tol = sqrt(p) * eps, the
// threshold of LAPACK's one-sided Jacobi (dgesvj): below it the inner products
// are rounding of the columns' own accuracy, and rotating on them only feeds
// back rounding
constexpr double SVD_EPS = 2.220446049250313e-16;
constexpr int SVD_ROUND_THREADS = 256;   // 8 warps, one column pair each
constexpr int SVD_FIN_THREADS = 512;
constexpr int SVD_SORT_MAX = 4096;       // columns per block the finishing sort holds
constexpr int64_t SVD_PANEL_SMEM = 200 * 1024;   // shared bytes of two panels of W and of V
constexpr int CUT_THREADS = 1024;
constexpr int CUT_MAX = 16384;           // values the device cut sorts in shared memory

struct SvdBlk {
    int64_t src_off;     // m x n source block, column-major, ld = m
    int64_t w_off;       // W (p x q, ld = p) in the workspace
    int64_t v_off;       // V (q x q, ld = q) in the workspace
    int64_t s_off;       // k = q singular values in S
    int64_t u_off;       // U: m x k, ld = m
    int64_t vt_off;      // Vt: k x n, ld = k
    int64_t pair_base;   // first pair of this block in a round's flat pair list
    int32_t m, n, p, q, qpad, trans;
    int64_t ppair_base;  // panel rounds: first panel pair of this block in a round's list
    int32_t nb, nbpad;   // panel rounds: panels of bw columns, rounded up to even
};

// per-block state: done flag and rotation counters of three consecutive sweeps
struct SvdState {
    int32_t done;
    int32_t sweeps;
    int32_t rot[3];
    int32_t pad;
};

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// W <- the block (or its transpose), V <- I
__global__ void svd_init_kernel(const SvdBlk* __restrict__ blks, const double* __restrict__ src,
                                double* __restrict__ work, SvdState* __restrict__ st) {
    const SvdBlk b = blks[blockIdx.y];
    const int64_t nw = (int64_t)b.p * b.q, nv = (int64_t)b.q * b.q;
    for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < nw + nv; e += (int64_t)gridDim.x * blockDim.x) {
        if (e < nw) {
            const int64_t r = e % b.p, c = e / b.p;
            // W(r, c) = A(r, c) or A(c, r)
            work[b.w_off + e] = b.trans ? src[b.src_off + c + r * b.m] : src[b.src_off + r + c * b.m];
        } else {
            const int64_t f = e - nw;
            work[b.v_off + f] = (f % b.q == f / b.q) ? 1.0 : 0.0;
        }
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        SvdState s;
        s.done = (b.q <= 1) ? 1 : 0;
        s.sweeps = 0;
        s.rot[0] = s.rot[1] = 0;
        s.rot[2] = 1;   // "sweep -1 rotated": sweep 0 always runs
        s.pad = 0;
        st[blockIdx.y] = s;
    }
}

// One tournament round for every unfinished block: g is the global round
// counter; block b is in sweep g / (qpad - 1), local round g % (qpad - 1).
__global__ void __launch_bounds__(SVD_ROUND_THREADS)
svd_round_kernel(const SvdBlk* __restrict__ blks, const int32_t* __restrict__ pair_blk, int64_t n_pairs,
                 double* __restrict__ work, SvdState* __restrict__ st, int32_t* __restrict__ remaining,
                 int32_t* __restrict__ status, int64_t g) {
    const int64_t wid = ((int64_t)blockIdx.x * SVD_ROUND_THREADS + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= n_pairs) return;
    const int bi = pair_blk[wid];
    const SvdBlk b = blks[bi];
    SvdState& s = st[bi];
    if (*(volatile int32_t*)&s.done) return;
    const int64_t R = b.qpad - 1;
    const int64_t r = g % R, sweep = g / R;
    const int64_t pidx = wid - b.pair_base;
    if (r == 0) {
        // the previous sweep's rotation count is final (written by earlier launches)
        const bool converged = sweep > 0 && s.rot[(sweep + 2) % 3] == 0;
        const bool exhausted = sweep >= SVD_MAX_SWEEPS;
        if (converged || exhausted) {
            if (pidx == 0 && lane == 0) {
                s.done = 1;
                s.sweeps = (int32_t)sweep;
                atomicSub(remaining, 1);
                if (!converged) atomicMax(status, bi + 1);
            }
            return;
        }
        // the counter of the next sweep was last written two sweeps ago
        if (pidx == 0 && lane == 0) s.rot[(sweep + 1) % 3] = 0;
    }
    // seats of the circle method: seat 0 fixed, the others rotate by r
    auto seat = [&](int64_t k) -> int64_t { return k == 0 ? 0 : 1 + (k - 1 + r) % R; };
    int64_t i = seat(pidx), j = seat(b.qpad - 1 - pidx);
    if (i > j) { const int64_t t = i; i = j; j = t; }
    if (j >= b.q) return;   // pair with the padding column
    double* __restrict__ wi = work + b.w_off + i * b.p;
    double* __restrict__ wj = work + b.w_off + j * b.p;
    double al = 0.0, be = 0.0, ga = 0.0;
    for (int64_t e = lane; e < b.p; e += 32) {
        const double x = wi[e], y = wj[e];
        al = fma(x, x, al);
        be = fma(y, y, be);
        ga = fma(x, y, ga);
    }
    al = warp_sum(al);
    be = warp_sum(be);
    ga = warp_sum(ga);
    if (ga == 0.0 || fabs(ga) <= sqrt((double)b.p) * SVD_EPS * sqrt(al) * sqrt(be)) return;
    const double zeta = (be - al) / (2.0 * ga);
    const double t = copysign(1.0, zeta) / (fabs(zeta) + hypot(1.0, zeta));
    const double c = 1.0 / sqrt(fma(t, t, 1.0));
    const double sn = c * t;
    for (int64_t e = lane; e < b.p; e += 32) {
        const double x = wi[e], y = wj[e];
        wi[e] = c * x - sn * y;
        wj[e] = sn * x + c * y;
    }
    double* __restrict__ vi = work + b.v_off + i * b.q;
    double* __restrict__ vj = work + b.v_off + j * b.q;
    for (int64_t e = lane; e < b.q; e += 32) {
        const double x = vi[e], y = vj[e];
        vi[e] = c * x - sn * y;
        vj[e] = sn * x + c * y;
    }
    if (lane == 0) atomicAdd(&s.rot[sweep % 3], 1);
}

// One round of the panel tournament for every unfinished block (see the file comment):
// CTA = one pair (I, J) of panels of bw columns, 32 bw threads; shared memory holds
// the 2 bw columns of W (ld = ldx >= p) and of V (ld = ldv >= q).  Every column pair
// of a block is rotated once per sweep, as in the single-column rounds: the cross
// pairs (a of I, b of J) in each round, bw inner rounds of the cyclic shift b = a + rr,
// warp a owning pair a; the pairs inside a panel in the first round of a sweep, a
// round-robin of bw - 1 inner rounds over each of I and J (warps 0 .. bw/2 - 1 on I,
// the others on J).  The same rotation (fresh inner products, the same threshold),
// applied to the W and V columns in shared memory; the columns go back if any rotated.
__global__ void svd_panel_round_kernel(const SvdBlk* __restrict__ blks, const int32_t* __restrict__ pair_blk,
                                       int64_t n_pairs, double* __restrict__ work, SvdState* __restrict__ st,
                                       int32_t* __restrict__ remaining, int32_t* __restrict__ status, int64_t g,
                                       int bw, int ldx, int ldv) {
    extern __shared__ double smem[];
    __shared__ int s_flag;
    const int64_t cta = blockIdx.x;
    if (cta >= n_pairs) return;
    const int bi = pair_blk[cta];
    const SvdBlk b = blks[bi];
    SvdState& s = st[bi];
    if (threadIdx.x == 0) s_flag = *(volatile int32_t*)&s.done;
    __syncthreads();
    if (s_flag) return;
    const int64_t R = b.nbpad - 1;
    const int64_t r = g % R, sweep = g / R;
    const int64_t pidx = cta - b.ppair_base;
    if (r == 0) {
        // the previous sweep's rotation count is final (written by earlier launches)
        const bool converged = sweep > 0 && s.rot[(sweep + 2) % 3] == 0;
        const bool exhausted = sweep >= SVD_MAX_SWEEPS;
        if (converged || exhausted) {
            if (pidx == 0 && threadIdx.x == 0) {
                s.done = 1;
                s.sweeps = (int32_t)sweep;
                atomicSub(remaining, 1);
                if (!converged) atomicMax(status, bi + 1);
            }
            return;
        }
        if (pidx == 0 && threadIdx.x == 0) s.rot[(sweep + 1) % 3] = 0;
    }
    auto seat = [&](int64_t k) -> int64_t { return k == 0 ? 0 : 1 + (k - 1 + r) % R; };
    int64_t I = seat(pidx), J = seat(b.nbpad - 1 - pidx);
    if (I > J) { const int64_t t = I; I = J; J = t; }
    const int nc = 2 * bw, p = b.p, q = b.q;
    // local column c: column I bw + c of the first panel or J bw + c - bw of the second;
    // columns at or past q (the padding panel, the last panel's tail) are absent
    auto gcol = [&](int c) -> int64_t { return c < bw ? I * bw + c : J * bw + (c - bw); };
    auto valid = [&](int c) -> bool { return gcol(c) < q; };
    double* sX = smem;
    double* sV = smem + (size_t)nc * ldx;
    for (int c = 0; c < nc; ++c) {
        const bool ok = valid(c);
        const double* src = work + b.w_off + (ok ? gcol(c) : 0) * (int64_t)p;
        for (int e = threadIdx.x; e < p; e += blockDim.x) sX[(size_t)c * ldx + e] = ok ? src[e] : 0.0;
        const double* vsrc = work + b.v_off + (ok ? gcol(c) : 0) * (int64_t)q;
        for (int e = threadIdx.x; e < q; e += blockDim.x) sV[(size_t)c * ldv + e] = ok ? vsrc[e] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x == 0) s_flag = 0;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double thr = sqrt((double)p) * SVD_EPS;
    bool rotated = false;
    auto rotate = [&](int i, int j) {
        double* __restrict__ xi = sX + (size_t)i * ldx;
        double* __restrict__ xj = sX + (size_t)j * ldx;
        double al = 0.0, be = 0.0, ga = 0.0;
        for (int e = lane; e < p; e += 32) {
            const double x = xi[e], y = xj[e];
            al = fma(x, x, al);
            be = fma(y, y, be);
            ga = fma(x, y, ga);
        }
        al = warp_sum(al);
        be = warp_sum(be);
        ga = warp_sum(ga);
        if (ga == 0.0 || fabs(ga) <= thr * sqrt(al) * sqrt(be)) return;
        const double zeta = (be - al) / (2.0 * ga);
        const double t = copysign(1.0, zeta) / (fabs(zeta) + hypot(1.0, zeta));
        const double c = 1.0 / sqrt(fma(t, t, 1.0));
        const double sn = c * t;
        for (int e = lane; e < p; e += 32) {
            const double x = xi[e], y = xj[e];
            xi[e] = c * x - sn * y;
            xj[e] = sn * x + c * y;
        }
        double* __restrict__ vi = sV + (size_t)i * ldv;
        double* __restrict__ vj = sV + (size_t)j * ldv;
        for (int e = lane; e < q; e += 32) {
            const double x = vi[e], y = vj[e];
            vi[e] = c * x - sn * y;
            vj[e] = sn * x + c * y;
        }
        rotated = true;
    };
    if (r == 0 && bw > 1) {
        // pairs inside each panel: warps [0, bw/2) on I, [bw/2, bw) on J
        const int half = bw / 2, side = warp / half, k = warp % half, Rw = bw - 1;
        for (int rr = 0; rr < Rw; ++rr) {
            const int k1 = bw - 1 - k;
            int i = k == 0 ? 0 : 1 + (k - 1 + rr) % Rw;
            int j = 1 + (k1 - 1 + rr) % Rw;
            if (i > j) { const int t = i; i = j; j = t; }
            i += side * bw;
            j += side * bw;
            if (valid(i) && valid(j)) rotate(i, j);
            __syncthreads();
        }
    }
    // cross pairs: warp a rotates (a, bw + (a + rr) % bw)
    for (int rr = 0; rr < bw; ++rr) {
        const int i = warp, j = bw + (warp + rr) % bw;
        if (valid(i) && valid(j)) rotate(i, j);
        __syncthreads();
    }
    if (rotated && lane == 0) s_flag = 1;
    __syncthreads();
    if (!s_flag) return;
    for (int c = 0; c < nc; ++c) {
        if (!valid(c)) continue;
        double* dst = work + b.w_off + gcol(c) * (int64_t)p;
        for (int e = threadIdx.x; e < p; e += blockDim.x) dst[e] = sX[(size_t)c * ldx + e];
        double* vdst = work + b.v_off + gcol(c) * (int64_t)q;
        for (int e = threadIdx.x; e < q; e += blockDim.x) vdst[e] = sV[(size_t)c * ldv + e];
    }
    if (threadIdx.x == 0) atomicAdd(&s.rot[sweep % 3], 1);
}

// Column norms, descending sort, and U / S / Vt in gesvd's layout.
__global__ void __launch_bounds__(SVD_FIN_THREADS)
svd_finish_kernel(const SvdBlk* __restrict__ blks, const double* __restrict__ work, double* __restrict__ U,
                  double* __restrict__ S, double* __restrict__ Vt) {
    __shared__ double sv[SVD_SORT_MAX];
    __shared__ int32_t si[SVD_SORT_MAX];
    const SvdBlk b = blks[blockIdx.x];
    const int q = b.q;
    if (q == 0) return;
    int np2 = 1;
    while (np2 < q) np2 <<= 1;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = SVD_FIN_THREADS / 32;
    for (int c = warp; c < np2; c += nwarps) {
        double a = 0.0;
        if (c < q) {
            const double* w = work + b.w_off + (int64_t)c * b.p;
            for (int64_t e = lane; e < b.p; e += 32) a = fma(w[e], w[e], a);
            a = warp_sum(a);
        }
        if (lane == 0) {
            sv[c] = c < q ? sqrt(a) : -1.0;
            si[c] = c;
        }
    }
    __syncthreads();
    // bitonic sort: descending value, ascending column on ties
    for (int k = 2; k <= np2; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int t = threadIdx.x; t < np2; t += SVD_FIN_THREADS) {
                const int o = t ^ jj;
                if (o > t) {
                    const bool first_before = (sv[t] > sv[o]) || (sv[t] == sv[o] && si[t] < si[o]);
                    const bool up = (t & k) == 0;
                    if (up ? !first_before : first_before) {
                        const double dv = sv[t]; sv[t] = sv[o]; sv[o] = dv;
                        const int32_t di = si[t]; si[t] = si[o]; si[o] = di;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int t = threadIdx.x; t < q; t += SVD_FIN_THREADS) S[b.s_off + t] = sv[t];
    // U: m x k (ld m); Vt: k x n (ld k), k = q
    const int64_t k = q;
    if (!b.trans) {
        // A = W S^-1 . S . V^T: U[:, t] = W[:, c] / s, Vt[t, :] = V[:, c]^T
        for (int64_t e = threadIdx.x; e < (int64_t)b.m * k; e += SVD_FIN_THREADS) {
            const int64_t r = e % b.m, t = e / b.m;
            const double s = sv[t];
            const double w = work[b.w_off + (int64_t)si[t] * b.p + r];
            U[b.u_off + e] = s > 0.0 ? w / s : 0.0;
        }
        for (int64_t e = threadIdx.x; e < k * b.n; e += SVD_FIN_THREADS) {
            const int64_t t = e % k, col = e / k;
            Vt[b.vt_off + e] = work[b.v_off + (int64_t)si[t] * b.q + col];
        }
    } else {
        // A^T = W V^T  =>  A = V W^T: U[:, t] = V[:, c], Vt[t, :] = W[:, c]^T / s
        for (int64_t e = threadIdx.x; e < (int64_t)b.m * k; e += SVD_FIN_THREADS) {
            const int64_t r = e % b.m, t = e / b.m;
            U[b.u_off + e] = work[b.v_off + (int64_t)si[t] * b.q + r];
        }
        for (int64_t e = threadIdx.x; e < k * b.n; e += SVD_FIN_THREADS) {
            const int64_t t = e % k, col = e / k;
            const double s = sv[t];
            const double w = work[b.w_off + (int64_t)si[t] * b.p + col];
            Vt[b.vt_off + e] = s > 0.0 ? w / s : 0.0;
        }
    }
}

// The truncation cut over all values of a batch (see the file comment).
struct CutOut {
    double evalscut, smallest_ev, sum_all, sum_disc, sum2_all, sum2_disc;
    int64_t kept;
};

__device__ double block_sum_fixed(double v, double* red) {
    v = warp_sum(v);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (threadIdx.x < 32) {
        t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
        t = warp_sum(t);
    }
    return t;   // valid in thread 0
}

__global__ void __launch_bounds__(CUT_THREADS)
trunc_cut_kernel(const double* __restrict__ vals, int64_t n, const int64_t* __restrict__ blk_off, int32_t nblk,
                 int64_t Mmax, double cutoff, int64_t* __restrict__ keep, CutOut* __restrict__ out) {
    extern __shared__ double sorted[];
    __shared__ double red[32];
    __shared__ double s_cut;
    int np2 = 1;
    while (np2 < n) np2 <<= 1;
    for (int t = threadIdx.x; t < np2; t += CUT_THREADS) sorted[t] = t < n ? vals[t] : -INFINITY;
    __syncthreads();
    for (int k = 2; k <= np2; k <<= 1) {
        for (int jj = k >> 1; jj > 0; jj >>= 1) {
            for (int t = threadIdx.x; t < np2; t += CUT_THREADS) {
                const int o = t ^ jj;
                if (o > t) {
                    const bool up = (t & k) == 0;
                    const bool sw = up ? (sorted[t] < sorted[o]) : (sorted[t] > sorted[o]);
                    if (sw) { const double d = sorted[t]; sorted[t] = sorted[o]; sorted[o] = d; }
                }
            }
            __syncthreads();
        }
    }
    if (threadIdx.x == 0) {
        double cut = cutoff * sorted[0];
        if (n > Mmax) cut = fmax(cut, sorted[Mmax]);
        s_cut = cut;
    }
    __syncthreads();
    const double cut = s_cut;
    // fixed-order sums over the sorted values: thread t owns a contiguous run
    double a = 0.0, d = 0.0, a2 = 0.0, d2 = 0.0;
    const int64_t per = (n + CUT_THREADS - 1) / CUT_THREADS;
    for (int64_t e = threadIdx.x * per; e < min(n, (int64_t)(threadIdx.x + 1) * per); ++e) {
        const double v = sorted[e];
        a += v;
        a2 = fma(v, v, a2);
        if (v < cut) { d += v; d2 = fma(v, v, d2); }
    }
    a = block_sum_fixed(a, red);
    __syncthreads();
    d = block_sum_fixed(d, red);
    __syncthreads();
    a2 = block_sum_fixed(a2, red);
    __syncthreads();
    d2 = block_sum_fixed(d2, red);
    // keeps per block: the leading run of values >= cut (each block's values are descending)
    for (int bi = threadIdx.x; bi < nblk; bi += CUT_THREADS) {
        int64_t c = 0;
        for (int64_t e = blk_off[bi]; e < blk_off[bi + 1] && vals[e] >= cut; ++e) ++c;
        keep[bi] = c;
    }
    if (threadIdx.x == 0) {
        CutOut o;
        o.evalscut = cut;
        o.smallest_ev = cut / sorted[0];
        o.sum_all = a;
        o.sum_disc = d;
        o.sum2_all = a2;
        o.sum2_disc = d2;
        o.kept = 0;
        *out = o;
    }
}

}  // namespace qcm

// ------------------------------------------------------------------ C ABI
using namespace qcm;

struct qcm_svd {
    std::vector<SvdBlk> blks;
    std::vector<int32_t> pair_blk;
    int64_t work_elems = 0, u_elems = 0, s_elems = 0, vt_elems = 0, n_pairs = 0, max_rounds = 0;
    // panel rounds (bw > 0; 0: single column pairs)
    int32_t bw = 0, ldx = 0, ldv = 0;
    std::vector<int32_t> ppair_blk;
    int64_t n_ppairs = 0, max_prounds = 0;
    int32_t* d_ppair_blk = nullptr;
    SvdBlk* d_blks = nullptr;
    int32_t* d_pair_blk = nullptr;
    SvdState* d_state = nullptr;
    int32_t* d_ctl = nullptr;      // remaining, status
    int32_t h_ctl[2] = {0, 0};     // host copy
    int device = -1;
    int32_t last_sweeps = 0;
};

static void svd_free(qcm_svd* s) {
    if (!s) return;
    cudaFree(s->d_blks);
    cudaFree(s->d_pair_blk);
    cudaFree(s->d_ppair_blk);
    cudaFree(s->d_state);
    cudaFree(s->d_ctl);
}

// panel pair lists of every block with q > 1 (bw = 0: none, single column pairs run)
static void svd_set_panels(qcm_svd* s, int32_t bw) {
    s->bw = bw;
    s->ppair_blk.clear();
    s->n_ppairs = 0;
    s->max_prounds = 0;
    s->ldx = 0;
    s->ldv = 0;
    if (bw <= 0) return;
    int64_t pairs = 0, rounds = 0;
    for (size_t k = 0; k < s->blks.size(); ++k) {
        SvdBlk& b = s->blks[k];
        b.nb = (b.q + bw - 1) / bw;
        b.nbpad = b.nb + (b.nb & 1);
        b.ppair_base = pairs;
        if (b.q > 1) {
            for (int32_t p = 0; p < b.nbpad / 2; ++p) s->ppair_blk.push_back((int32_t)k);
            pairs += b.nbpad / 2;
            rounds = std::max<int64_t>(rounds, b.nbpad - 1);
            s->ldx = std::max<int32_t>(s->ldx, b.p);
            s->ldv = std::max<int32_t>(s->ldv, b.q);
        }
    }
    s->n_ppairs = pairs;
    s->max_prounds = rounds;
}

extern "C" {

int qcm_svd_create(int32_t nblocks, const int64_t* rows, const int64_t* cols, const int64_t* src_off, qcm_svd** out) {
    if (!out || nblocks < 0 || (nblocks > 0 && (!rows || !cols || !src_off))) {
        set_error("qcm_svd_create: invalid arguments");
        return QCM_E_INVALID;
    }
    *out = nullptr;
    auto* s = new qcm_svd();
    int64_t w = 0, u = 0, sv = 0, vt = 0, pairs = 0, rounds = 0;
    for (int32_t k = 0; k < nblocks; ++k) {
        if (rows[k] < 0 || cols[k] < 0 || src_off[k] < 0 || rows[k] > (1 << 30) || cols[k] > (1 << 30)) {
            delete s;
            set_error("qcm_svd_create: block " + std::to_string(k) + " has an invalid extent");
            return QCM_E_INVALID;
        }
        SvdBlk b;
        b.m = (int32_t)rows[k];
        b.n = (int32_t)cols[k];
        b.trans = b.m < b.n;
        b.p = b.trans ? b.n : b.m;
        b.q = b.trans ? b.m : b.n;
        if (b.q > SVD_SORT_MAX) {
            delete s;
            set_error("qcm_svd_create: block " + std::to_string(k) + " has min(rows, cols) = " + std::to_string(b.q) +
                      " > " + std::to_string(SVD_SORT_MAX));
            return QCM_E_RANGE;
        }
        b.qpad = b.q + (b.q & 1);
        b.src_off = src_off[k];
        b.w_off = w;
        w += (int64_t)b.p * b.q;
        b.v_off = w;
        w += (int64_t)b.q * b.q;
        b.s_off = sv;
        sv += b.q;
        b.u_off = u;
        u += (int64_t)b.m * b.q;
        b.vt_off = vt;
        vt += (int64_t)b.q * b.n;
        b.pair_base = pairs;
        if (b.q > 1) {
            for (int32_t p = 0; p < b.qpad / 2; ++p) s->pair_blk.push_back(k);
            pairs += b.qpad / 2;
            rounds = std::max<int64_t>(rounds, b.qpad - 1);
        }
        s->blks.push_back(b);
    }
    s->work_elems = w;
    s->u_elems = u;
    s->s_elems = sv;
    s->vt_elems = vt;
    s->n_pairs = pairs;
    s->max_rounds = rounds;
    // the widest panels whose two panels of W and of V fit in shared memory, if at
    // least 8 columns wide: narrower panels (tall blocks) leave one CTA of few warps per
    // SM and measured slower than single column pairs
    int64_t pmax = 0, qmax = 0;
    for (auto& b : s->blks)
        if (b.q > 1) { pmax = std::max<int64_t>(pmax, b.p); qmax = std::max<int64_t>(qmax, b.q); }
    int32_t bw = 0;
    for (int32_t cand : {16, 8})
        if (2 * cand * (pmax + qmax) * (int64_t)sizeof(double) <= SVD_PANEL_SMEM) { bw = cand; break; }
    svd_set_panels(s, bw);
    *out = s;
    return QCM_OK;
}

int qcm_svd_set_panel_width(qcm_svd* s, int32_t bw) {
    if (!s) { set_error("null svd"); return QCM_E_INVALID; }
    if (s->d_blks) { set_error("qcm_svd_set_panel_width: the factorisation has already run"); return QCM_E_STATE; }
    if (bw != 0 && bw != 2 && bw != 4 && bw != 8 && bw != 16) {
        set_error("qcm_svd_set_panel_width: width must be 0, 2, 4, 8 or 16");
        return QCM_E_INVALID;
    }
    int64_t pmax = 0, qmax = 0;
    for (auto& b : s->blks)
        if (b.q > 1) { pmax = std::max<int64_t>(pmax, b.p); qmax = std::max<int64_t>(qmax, b.q); }
    if (bw > 0 && 2 * bw * (pmax + qmax) * (int64_t)sizeof(double) > SVD_PANEL_SMEM) {
        set_error("qcm_svd_set_panel_width: two panels of the tallest block exceed shared memory");
        return QCM_E_RANGE;
    }
    svd_set_panels(s, bw);
    return QCM_OK;
}

int qcm_svd_panel_width(const qcm_svd* s, int32_t* bw) {
    if (!s || !bw) { set_error("null argument"); return QCM_E_INVALID; }
    *bw = s->bw;
    return QCM_OK;
}

int qcm_svd_sizes(const qcm_svd* s, int64_t* work_elems, int64_t* u_elems, int64_t* s_elems, int64_t* vt_elems) {
    if (!s) { set_error("null svd"); return QCM_E_INVALID; }
    if (work_elems) *work_elems = s->work_elems;
    if (u_elems) *u_elems = s->u_elems;
    if (s_elems) *s_elems = s->s_elems;
    if (vt_elems) *vt_elems = s->vt_elems;
    return QCM_OK;
}

int qcm_svd_block_offsets(const qcm_svd* s, int64_t* s_off, int64_t* u_off, int64_t* vt_off) {
    if (!s) { set_error("null svd"); return QCM_E_INVALID; }
    for (size_t k = 0; k < s->blks.size(); ++k) {
        if (s_off) s_off[k] = s->blks[k].s_off;
        if (u_off) u_off[k] = s->blks[k].u_off;
        if (vt_off) vt_off[k] = s->blks[k].vt_off;
    }
    return QCM_OK;
}

int qcm_svd_run(qcm_svd* s, const double* src, double* work, double* U, double* S, double* Vt, void* stream) {
    if (!s) { set_error("null svd"); return QCM_E_INVALID; }
    if (s->blks.empty()) return QCM_OK;
    if (!src || !work || !U || !S || !Vt) { set_error("qcm_svd_run: null buffer"); return QCM_E_INVALID; }
    int dev = 0;
    FCT_CUDA(cudaGetDevice(&dev));
    if (!s->d_blks) {
        FCT_CUDA(cudaMalloc(&s->d_blks, sizeof(SvdBlk) * s->blks.size()));
        FCT_CUDA(cudaMemcpy(s->d_blks, s->blks.data(), sizeof(SvdBlk) * s->blks.size(), cudaMemcpyHostToDevice));
        if (!s->pair_blk.empty()) {
            FCT_CUDA(cudaMalloc(&s->d_pair_blk, sizeof(int32_t) * s->pair_blk.size()));
            FCT_CUDA(cudaMemcpy(s->d_pair_blk, s->pair_blk.data(), sizeof(int32_t) * s->pair_blk.size(),
                                cudaMemcpyHostToDevice));
        }
        if (!s->ppair_blk.empty()) {
            FCT_CUDA(cudaMalloc(&s->d_ppair_blk, sizeof(int32_t) * s->ppair_blk.size()));
            FCT_CUDA(cudaMemcpy(s->d_ppair_blk, s->ppair_blk.data(), sizeof(int32_t) * s->ppair_blk.size(),
                                cudaMemcpyHostToDevice));
        }
        FCT_CUDA(cudaMalloc(&s->d_state, sizeof(SvdState) * s->blks.size()));
        FCT_CUDA(cudaMalloc(&s->d_ctl, sizeof(int32_t) * 2));
        s->device = dev;
    } else if (dev != s->device) {
        set_error("qcm_svd_run: the factorisation was set up on another device");
        return QCM_E_STATE;
    }
    cudaStream_t st = (cudaStream_t)stream;
    int32_t active = 0;
    for (auto& b : s->blks) active += b.q > 1;
    int32_t ctl0[2] = {active, 0};
    FCT_CUDA(cudaMemcpyAsync(s->d_ctl, ctl0, sizeof(ctl0), cudaMemcpyHostToDevice, st));
    const int64_t maxel = [&] {
        int64_t mx = 1;
        for (auto& b : s->blks) mx = std::max<int64_t>(mx, (int64_t)b.p * b.q + (int64_t)b.q * b.q);
        return mx;
    }();
    dim3 ig((unsigned)std::min<int64_t>((maxel + 255) / 256, 1024), (unsigned)s->blks.size());
    svd_init_kernel<<<ig, 256, 0, st>>>(s->d_blks, src, work, s->d_state);
    FCT_CUDA(cudaGetLastError());
    int64_t g = 0;
    s->last_sweeps = 0;
    if (active > 0) {
        const unsigned grid = (unsigned)((s->n_pairs * 32 + SVD_ROUND_THREADS - 1) / SVD_ROUND_THREADS);
        const size_t psmem = (size_t)(2 * s->bw * ((int64_t)s->ldx + s->ldv)) * sizeof(double);
        if (s->bw > 0)
            FCT_CUDA(cudaFuncSetAttribute(svd_panel_round_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                          (int)psmem));
        const int64_t rounds = s->bw > 0 ? s->max_prounds : s->max_rounds;
        // rounds in chunks of one sweep of the widest block; then ask whether any block is left
        for (int chunk = 0; chunk <= SVD_MAX_SWEEPS + 1; ++chunk) {
            for (int64_t r = 0; r < rounds; ++r, ++g) {
                if (s->bw > 0)
                    svd_panel_round_kernel<<<(unsigned)s->n_ppairs, 32 * s->bw, psmem, st>>>(
                        s->d_blks, s->d_ppair_blk, s->n_ppairs, work, s->d_state, s->d_ctl, s->d_ctl + 1, g, s->bw,
                        s->ldx, s->ldv);
                else
                    svd_round_kernel<<<grid, SVD_ROUND_THREADS, 0, st>>>(s->d_blks, s->d_pair_blk, s->n_pairs, work,
                                                                         s->d_state, s->d_ctl, s->d_ctl + 1, g);
            }
            FCT_CUDA(cudaGetLastError());
            FCT_CUDA(cudaMemcpyAsync(s->h_ctl, s->d_ctl, sizeof(int32_t) * 2, cudaMemcpyDeviceToHost, st));
            FCT_CUDA(cudaStreamSynchronize(st));
            s->last_sweeps = chunk + 1;
            if (s->h_ctl[0] <= 0) break;
        }
    }
    svd_finish_kernel<<<(unsigned)s->blks.size(), SVD_FIN_THREADS, 0, st>>>(s->d_blks, work, U, S, Vt);
    FCT_CUDA(cudaGetLastError());
    if (active > 0 && (s->h_ctl[0] > 0 || s->h_ctl[1] != 0)) {
        set_error("qcm_svd_run: block " + std::to_string(s->h_ctl[1] > 0 ? s->h_ctl[1] - 1 : -1) +
                  " did not converge in " + std::to_string(SVD_MAX_SWEEPS) + " sweeps");
        return QCM_E_RANGE;
    }
    return QCM_OK;
}

int qcm_svd_last_sweeps(const qcm_svd* s, int32_t* chunks) {
    if (!s || !chunks) { set_error("null argument"); return QCM_E_INVALID; }
    *chunks = s->last_sweeps;
    return QCM_OK;
}

void qcm_svd_destroy(qcm_svd* s) {
    svd_free(s);
    delete s;
}

int qcm_truncation_cut(const double* vals_dev, int32_t nblocks, const int64_t* blk_off, int64_t Mmax, double cutoff,
                       int32_t mode, int64_t* keep, qcm_trunc_t* out, void* stream) {
    if (nblocks < 0 || !blk_off || !keep || !out || (nblocks > 0 && !vals_dev)) {
        set_error("qcm_truncation_cut: invalid arguments");
        return QCM_E_INVALID;
    }
    const int64_t n = nblocks > 0 ? blk_off[nblocks] : 0;
    std::memset(out, 0, sizeof(*out));
    if (n == 0) {
        for (int32_t k = 0; k < nblocks; ++k) keep[k] = 0;
        return QCM_OK;
    }
    if (n > CUT_MAX) {
        set_error("qcm_truncation_cut: " + std::to_string(n) + " values exceed the device cut's capacity of " +
                  std::to_string(CUT_MAX));
        return QCM_E_RANGE;
    }
    if (Mmax < 0) { set_error("qcm_truncation_cut: negative Mmax"); return QCM_E_INVALID; }
    cudaStream_t st = (cudaStream_t)stream;
    int64_t* d_off = nullptr;
    int64_t* d_keep = nullptr;
    CutOut* d_out = nullptr;
    FCT_CUDA(cudaMallocAsync(&d_off, sizeof(int64_t) * (nblocks + 1), st));
    FCT_CUDA(cudaMallocAsync(&d_keep, sizeof(int64_t) * std::max(nblocks, 1), st));
    FCT_CUDA(cudaMallocAsync(&d_out, sizeof(CutOut), st));
    FCT_CUDA(cudaMemcpyAsync(d_off, blk_off, sizeof(int64_t) * (nblocks + 1), cudaMemcpyHostToDevice, st));
    int np2 = 1;
    while (np2 < n) np2 <<= 1;
    const size_t smem = sizeof(double) * np2;
    if (smem > 48 * 1024) FCT_CUDA(cudaFuncSetAttribute(trunc_cut_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                        (int)smem));
    trunc_cut_kernel<<<1, CUT_THREADS, smem, st>>>(vals_dev, n, d_off, nblocks, Mmax, cutoff, d_keep, d_out);
    FCT_CUDA(cudaGetLastError());
    CutOut h;
    FCT_CUDA(cudaMemcpyAsync(keep, d_keep, sizeof(int64_t) * nblocks, cudaMemcpyDeviceToHost, st));
    FCT_CUDA(cudaMemcpyAsync(&h, d_out, sizeof(CutOut), cudaMemcpyDeviceToHost, st));
    FCT_CUDA(cudaFreeAsync(d_off, st));
    FCT_CUDA(cudaFreeAsync(d_keep, st));
    FCT_CUDA(cudaFreeAsync(d_out, st));
    FCT_CUDA(cudaStreamSynchronize(st));
    int64_t kept = 0;
    for (int32_t k = 0; k < nblocks; ++k) kept += keep[k];
    out->bond_dimension = kept;
    out->evalscut = h.evalscut;
    out->smallest_ev = h.smallest_ev;
    out->truncated_fraction = h.sum_all > 0.0 ? h.sum_disc / h.sum_all : 0.0;
    // mode 0 (singular values): weight = sum of discarded s^2 / sum of s^2;
    // mode 1 (density-matrix eigenvalues): the reference reports the fraction in both fields
    out->truncated_weight = mode == 0 ? (h.sum2_all > 0.0 ? h.sum2_disc / h.sum2_all : 0.0) : out->truncated_fraction;
    return QCM_OK;
}

}  // extern "C"
