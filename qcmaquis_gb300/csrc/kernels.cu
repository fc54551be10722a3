// Device executors for contraction plans and the FP64 vector kernels of the
// eigensolver.  Compiled for sm_103a only.
//
// * gather_axpy_kernel   -- the lbtm/rbtm micro-axpys (ct/non-abelian/micro_kernels.hpp:19-198)
//   regrouped per output tile: each work item owns one column range of one
//   output tile and writes it once (sum of scaled source stripes, fixed order).
// * gemm_f64_kernel      -- grouped, segmented FP64 block products (the dgemm calls
//   of ct/non-abelian/gemm.hpp:48-204): every work item owns one 64x64 output
//   tile and sums all its segments (split-K over MPO bond indices) in registers.
// * dot/nrm2/axpby/...   -- ietl::dot / two_norm / vector updates of the
//   Jacobi-Davidson loop (dmrg/framework/ietl/jacobi.h:385-435), with
//   deterministic two-pass reductions (warp shuffles, fixed combine order).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <numeric>
#include <string>
#include <unordered_map>
#include <vector>

#include "plan.hpp"


namespace qcm {

#define QCM_CUDA(call)                                                                  \
    do {                                                                                \
        cudaError_t err__ = (call);                                                     \
        if (err__ != cudaSuccess) {                                                     \
            set_error(std::string(#call) + ": " + cudaGetErrorString(err__));           \
            return QCM_E_CUDA;                                                          \
        }                                                                               \
    } while (0)

struct DevAxpyOut { int64_t dst_off, ldd, rows, cols, t_begin, t_end; int32_t dst_buf, pad; };  // pad: pitch
struct DevAxpyTerm { int64_t src_off, lds; double alpha; int32_t src_buf, pad; };
struct DevAxpyWork { int64_t out, c0, c1; };
struct DevAxpyChunk { int32_t out, e0, n, pad; };
struct DevGemmOut { int64_t c_off, ldc, M, N, s_begin, s_end; int32_t c_buf, pad; };
struct DevGemmSeg { int64_t a_off, lda, b_off, ldb, K; double alpha; int32_t a_buf, ta, b_buf, tb; };
struct DevGemmWork { int64_t out, m0, n0; int32_t tm, tn; };   // tile extents: tm % 16 == 0, tn % 32 == 0

// Buffer table of one plan run.  Bit i of f32mask marks slot i as FP32 (the
// mixed-precision forms keep boundary shadows and all intermediates in FP32);
// every other slot holds FP64.
struct BufTable { double* p[QCM_NBUF]; uint32_t f32mask; };

__device__ __forceinline__ bool slot_f32(const BufTable& b, int slot) { return (b.f32mask >> slot) & 1u; }

// ------------------------------------------------------------------ gather-axpy
constexpr int AXPY_THREADS = 256;
constexpr int AXPY_TERM_CACHE = 128;

// ACC = double for the FP64 form, float for the mixed forms (FP32 intermediates).
template <class ACC>
__global__ void __launch_bounds__(AXPY_THREADS)
gather_axpy_kernel(BufTable bufs, const DevAxpyOut* __restrict__ outs, const DevAxpyTerm* __restrict__ terms,
                   const DevAxpyWork* __restrict__ work) {
    __shared__ ACC s_alpha[AXPY_TERM_CACHE];
    __shared__ const void* s_src[AXPY_TERM_CACHE];
    __shared__ int64_t s_lds[AXPY_TERM_CACHE];
    __shared__ int s_f32[AXPY_TERM_CACHE];
    const DevAxpyWork w = work[blockIdx.x];
    const DevAxpyOut o = outs[w.out];
    const bool dst32 = slot_f32(bufs, o.dst_buf);
    const int64_t rows = o.rows;
    const int64_t nel = rows * (w.c1 - w.c0);
    const int64_t nterm = o.t_end - o.t_begin;
    for (int64_t base = 0; base < nel; base += 4 * AXPY_THREADS) {
        ACC acc[4] = {ACC(0), ACC(0), ACC(0), ACC(0)};
        int64_t ii[4], jj[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int64_t e = base + threadIdx.x + (int64_t)u * AXPY_THREADS;
            ii[u] = e % rows;
            jj[u] = w.c0 + e / rows;
        }
        for (int64_t t0 = 0; t0 < nterm; t0 += AXPY_TERM_CACHE) {
            const int64_t tn = min((int64_t)AXPY_TERM_CACHE, nterm - t0);
            __syncthreads();
            for (int64_t t = threadIdx.x; t < tn; t += AXPY_THREADS) {
                const DevAxpyTerm tt = terms[o.t_begin + t0 + t];
                const bool f32 = slot_f32(bufs, tt.src_buf);
                s_alpha[t] = (ACC)tt.alpha;
                s_src[t] = f32 ? (const void*)((const float*)bufs.p[tt.src_buf] + tt.src_off)
                               : (const void*)(bufs.p[tt.src_buf] + tt.src_off);
                s_lds[t] = tt.lds;
                s_f32[t] = f32 ? 1 : 0;
            }
            __syncthreads();
            for (int64_t t = 0; t < tn; ++t) {
                const ACC a = s_alpha[t];
                const int64_t lds = s_lds[t];
                if (s_f32[t]) {
                    const float* __restrict__ src = (const float*)s_src[t];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        int64_t e = base + threadIdx.x + (int64_t)u * AXPY_THREADS;
                        if (e < nel) acc[u] = fma(a, (ACC)__ldg(src + ii[u] + jj[u] * lds), acc[u]);
                    }
                } else {
                    const double* __restrict__ src = (const double*)s_src[t];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        int64_t e = base + threadIdx.x + (int64_t)u * AXPY_THREADS;
                        if (e < nel) acc[u] = fma(a, (ACC)__ldg(src + ii[u] + jj[u] * lds), acc[u]);
                    }
                }
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int64_t e = base + threadIdx.x + (int64_t)u * AXPY_THREADS;
            if (e < nel) {
                if (dst32) ((float*)bufs.p[o.dst_buf])[o.dst_off + ii[u] + jj[u] * o.ldd] = (float)acc[u];
                else bufs.p[o.dst_buf][o.dst_off + ii[u] + jj[u] * o.ldd] = (double)acc[u];
            }
        }
    }
}

// Fast path for stages whose terms all read buffers of one element type SRC:
// term loop unrolled by 4 so that 16 independent loads per thread are in flight
// (the gathers re-read their sources mostly from L2 and are latency bound).
template <class ACC, class SRC>
__global__ void __launch_bounds__(AXPY_THREADS)
gather_axpy_uniform(BufTable bufs, const DevAxpyOut* __restrict__ outs, const DevAxpyTerm* __restrict__ terms,
                    const DevAxpyWork* __restrict__ work) {
    __shared__ ACC s_alpha[AXPY_TERM_CACHE];
    __shared__ const SRC* s_src[AXPY_TERM_CACHE];
    __shared__ int s_lds[AXPY_TERM_CACHE];
    const DevAxpyWork w = work[blockIdx.x];
    const DevAxpyOut o = outs[w.out];
    const bool dst32 = slot_f32(bufs, o.dst_buf);
    const int64_t rows = o.rows;
    const int64_t nel = rows * (w.c1 - w.c0);
    const int64_t nterm = o.t_end - o.t_begin;
    for (int64_t base = 0; base < nel; base += 4 * AXPY_THREADS) {
        ACC acc[4] = {ACC(0), ACC(0), ACC(0), ACC(0)};
        int ii[4], jj[4];  // in-tile row and column (tiles are far below 2^31 elements)
        bool ok[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            int64_t e = base + threadIdx.x + (int64_t)u * AXPY_THREADS;
            ok[u] = e < nel;
            ii[u] = ok[u] ? (int)(e % rows) : 0;
            jj[u] = ok[u] ? (int)(w.c0 + e / rows) : (int)w.c0;
        }
        for (int64_t t0 = 0; t0 < nterm; t0 += AXPY_TERM_CACHE) {
            const int64_t tn = min((int64_t)AXPY_TERM_CACHE, nterm - t0);
            __syncthreads();
            for (int64_t t = threadIdx.x; t < tn; t += AXPY_THREADS) {
                const DevAxpyTerm tt = terms[o.t_begin + t0 + t];
                s_alpha[t] = (ACC)tt.alpha;
                s_src[t] = (const SRC*)bufs.p[tt.src_buf] + tt.src_off;
                s_lds[t] = (int)tt.lds;
            }
            __syncthreads();
            int64_t t = 0;
            for (; t + 4 <= tn; t += 4) {
                SRC x[4][4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const SRC* __restrict__ src = s_src[t + q];
                    const int lds = s_lds[t + q];
#pragma unroll
                    for (int u = 0; u < 4; ++u) x[q][u] = ok[u] ? __ldg(src + ii[u] + jj[u] * lds) : SRC(0);
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const ACC a = s_alpha[t + q];
#pragma unroll
                    for (int u = 0; u < 4; ++u) acc[u] = fma(a, (ACC)x[q][u], acc[u]);
                }
            }
            for (; t < tn; ++t) {
                const SRC* __restrict__ src = s_src[t];
                const int lds = s_lds[t];
                const ACC a = s_alpha[t];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (ok[u]) acc[u] = fma(a, (ACC)__ldg(src + ii[u] + jj[u] * lds), acc[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            if (ok[u]) {
                const int64_t d = o.dst_off + ii[u] + (int64_t)jj[u] * o.ldd;
                if (dst32) ((float*)bufs.p[o.dst_buf])[d] = (float)acc[u];
                else bufs.p[o.dst_buf][d] = (double)acc[u];
            }
        }
    }
}

// Contiguous-source executor.  Every term of an output tile reads a source tile
// stored contiguously with one pitch (its leading dimension: rows, or rows
// rounded up to 4 elements for the 16-byte aligned K1 result), so element e of
// the tile's pitch x cols run is sum_t alpha_t * src_t[e] over the tile's terms
// in order, and the elements of the padding rows (e % pitch >= rows) are never
// stored.  A work item owns CG_CHUNK consecutive elements of one tile; each
// thread keeps CG_PER accumulators and reads every source through one per-term
// pointer (cached in shared memory).  (Four-element vector loads over the
// 16-byte aligned K1 result were measured slower: 14.2 against 13.2 ms per
// sigma at the benchmark size.)
constexpr int CG_THREADS = 256;
constexpr int CG_PER = 8;
constexpr int CG_CHUNK = CG_THREADS * CG_PER;
constexpr int CG_TCACHE = 256;

template <class ACC, class SRC>
__global__ void __launch_bounds__(CG_THREADS)
gather_axpy_contig(BufTable bufs, const DevAxpyOut* __restrict__ outs, const DevAxpyTerm* __restrict__ terms,
                   const DevAxpyChunk* __restrict__ work) {
    __shared__ const SRC* s_ptr[CG_TCACHE];
    __shared__ ACC s_alpha[CG_TCACHE];
    const DevAxpyChunk w = work[blockIdx.x];
    const DevAxpyOut o = outs[w.out];
    const int tid = threadIdx.x;
    const int n = w.n;
    const int pitch = o.pad > 0 ? o.pad : (int)o.rows;
    ACC acc[CG_PER];
#pragma unroll
    for (int u = 0; u < CG_PER; ++u) acc[u] = ACC(0);
    const int64_t nterm = o.t_end - o.t_begin;
    for (int64_t t0 = 0; t0 < nterm; t0 += CG_TCACHE) {
        const int tn = (int)min((int64_t)CG_TCACHE, nterm - t0);
        __syncthreads();
        if (tid < tn) {
            const DevAxpyTerm tt = terms[o.t_begin + t0 + tid];
            s_ptr[tid] = (const SRC*)bufs.p[tt.src_buf] + tt.src_off + w.e0;
            s_alpha[tid] = (ACC)tt.alpha;
        }
        __syncthreads();
        if (n == CG_CHUNK) {
            int t = 0;
            for (; t + 2 <= tn; t += 2) {
                const SRC* __restrict__ p0 = s_ptr[t] + tid;
                const SRC* __restrict__ p1 = s_ptr[t + 1] + tid;
                SRC x0[CG_PER], x1[CG_PER];
#pragma unroll
                for (int u = 0; u < CG_PER; ++u) {
                    x0[u] = __ldg(p0 + u * CG_THREADS);
                    x1[u] = __ldg(p1 + u * CG_THREADS);
                }
                const ACC a0 = s_alpha[t], a1 = s_alpha[t + 1];
#pragma unroll
                for (int u = 0; u < CG_PER; ++u) {
                    acc[u] = fma(a0, (ACC)x0[u], acc[u]);
                    acc[u] = fma(a1, (ACC)x1[u], acc[u]);
                }
            }
            if (t < tn) {
                const SRC* __restrict__ p0 = s_ptr[t] + tid;
                const ACC a0 = s_alpha[t];
#pragma unroll
                for (int u = 0; u < CG_PER; ++u) acc[u] = fma(a0, (ACC)__ldg(p0 + u * CG_THREADS), acc[u]);
            }
        } else {
            // a short chunk: one term per iteration (four terms per iteration, with the
            // loads past n predicated off, measured slower: K2 6.29 against 5.86 ms)
            for (int t = 0; t < tn; ++t) {
                const SRC* __restrict__ p0 = s_ptr[t] + tid;
                const ACC a0 = s_alpha[t];
#pragma unroll
                for (int u = 0; u < CG_PER; ++u)
                    if (tid + u * CG_THREADS < n) acc[u] = fma(a0, (ACC)__ldg(p0 + u * CG_THREADS), acc[u]);
            }
        }
    }
    const bool dst32 = slot_f32(bufs, o.dst_buf);
    // element e of the run sits at row e % pitch, column e / pitch: one division
    // for the first element, then steps of CG_THREADS elements with a carry
    const int rows = (int)o.rows;
    const int e_first = w.e0 + tid;
    int rr = e_first % pitch, cc = e_first / pitch;
    const int dr = CG_THREADS % pitch, dc = CG_THREADS / pitch;
    float* __restrict__ D32 = (float*)bufs.p[o.dst_buf] + o.dst_off;
    double* __restrict__ D64 = bufs.p[o.dst_buf] + o.dst_off;
#pragma unroll
    for (int u = 0; u < CG_PER; ++u) {
        if (tid + u * CG_THREADS < n && rr < rows) {
            const int64_t d = rr + (int64_t)cc * o.ldd;
            if (dst32) D32[d] = (float)acc[u];
            else D64[d] = (double)acc[u];
        }
        rr += dr;
        cc += dc;
        if (rr >= pitch) { rr -= pitch; ++cc; }
    }
}

// Work list of the contiguous-source executor, ordered so that CTAs running
// at the same time read the same source chunks: output tiles that share a
// source tile (transitively) form one group; groups run one after another,
// and inside a group all tiles' chunk 0 runs before any chunk 1, and so on.
// Returns false (and no list) when some term's source is not contiguous.
// ------------------------------------------------------------------ adjoint (energy gradient)
// One term of a DOT stage: a source tile and the output-adjoint tile it pairs with.
struct DevDotTerm {
    int64_t src_off, lds, dst_off, ldd;
    int32_t rows, cols, src_buf, dst_buf;
};
constexpr int DOT_THREADS = 256;

// g[k] = sum over the tile of src_k * dst_k (FP64), one CTA per term at a time; the
// element order and the reduction tree are fixed, so the result is deterministic.
__global__ void __launch_bounds__(DOT_THREADS) dot_terms_kernel(BufTable bt, const DevDotTerm* __restrict__ terms,
                                                                int64_t n, double* __restrict__ g) {
    __shared__ double red[DOT_THREADS / 32];
    for (int64_t k = blockIdx.x; k < n; k += gridDim.x) {
        const DevDotTerm t = terms[k];
        const double* __restrict__ src = bt.p[t.src_buf] + t.src_off;
        const double* __restrict__ dst = bt.p[t.dst_buf] + t.dst_off;
        double acc = 0.0;
        if (t.rows >= 32) {
            // warps over columns, lanes down the column
            const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
            for (int c = warp; c < t.cols; c += DOT_THREADS / 32) {
                const double* sc = src + (int64_t)c * t.lds;
                const double* dc = dst + (int64_t)c * t.ldd;
                for (int r = lane; r < t.rows; r += 32) acc = fma(sc[r], dc[r], acc);
            }
        } else {
            const int64_t ne = (int64_t)t.rows * t.cols;
            for (int64_t e = threadIdx.x; e < ne; e += DOT_THREADS) {
                const int64_t c = e / t.rows, r = e - c * t.rows;
                acc = fma(src[r + c * t.lds], dst[r + c * t.ldd], acc);
            }
        }
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
        if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
        __syncthreads();
        if (threadIdx.x == 0) {
            double v = 0.0;
            for (int w = 0; w < DOT_THREADS / 32; ++w) v += red[w];
            g[k] = v;
        }
        __syncthreads();
    }
}

// out[tt] = sum over the terms of tt (ascending term index) of w[k] g[k]
__global__ void dot_reduce_kernel(const int64_t* __restrict__ ptr, const int64_t* __restrict__ idx,
                                  const double* __restrict__ w, const double* __restrict__ g, int32_t n_tt,
                                  double* __restrict__ out) {
    const int32_t tt = blockIdx.x * blockDim.x + threadIdx.x;
    if (tt >= n_tt) return;
    double acc = 0.0;
    for (int64_t q = ptr[tt]; q < ptr[tt + 1]; ++q) {
        const int64_t k = idx[q];
        acc = fma(w[k], g[k], acc);
    }
    out[tt] = acc;
}

static bool build_chunk_work(const Stage& st, std::vector<DevAxpyChunk>& w) {
    const size_t nO = st.aout.size();
    std::vector<int64_t> pitch(nO), nel(nO);
    for (size_t i = 0; i < nO; ++i) {
        const AxpyOut& a = st.aout[i];
        pitch[i] = tile_pitch(st, a);
        if (pitch[i] < 0 || a.rows <= 0 || pitch[i] * a.cols > 0x7fffffffLL) return false;
        nel[i] = pitch[i] * (a.cols - 1) + a.rows;
    }
    std::vector<int32_t> rootv;
    const std::vector<int32_t>* roots = &st.comp_root;
    if (st.comp_root.size() != nO) {
        if (!axpy_components(st, rootv)) return false;
        roots = &rootv;
    }
    // groups in order of their first output; members in output order
    std::vector<int32_t> order(nO);
    std::iota(order.begin(), order.end(), 0);
    const std::vector<int32_t>& root = *roots;
    std::stable_sort(order.begin(), order.end(), [&](int32_t x, int32_t y) { return root[x] < root[y]; });
    w.clear();
    for (size_t g0 = 0; g0 < nO;) {
        size_t g1 = g0;
        int64_t maxc = 0;
        while (g1 < nO && root[order[g1]] == root[order[g0]]) {
            maxc = std::max<int64_t>(maxc, (nel[order[g1]] + CG_CHUNK - 1) / CG_CHUNK);
            ++g1;
        }
        for (int64_t c = 0; c < maxc; ++c)
            for (size_t k = g0; k < g1; ++k) {
                const int64_t ne = nel[order[k]];
                if (c * CG_CHUNK < ne)
                    w.push_back({order[k], (int32_t)(c * CG_CHUNK), (int32_t)std::min<int64_t>(CG_CHUNK, ne - c * CG_CHUNK), 0});
            }
        g0 = g1;
    }
    return true;
}

// ------------------------------------------------------------------ FP64 grouped GEMM
constexpr int GT_M = 64, GT_N = 64, GT_K = 16;
constexpr int GT_LD = GT_M + 2;   // shared row stride: even (16-byte aligned two-double reads)

// One tile of a grouped FP64 product per CTA, of extent tm x tn (tm a multiple of
// 16, tn of 32, both at most 64: a block's last tiles are cut to its size, so
// that little of the FP64 work is spent on padding -- GB300's FP64 rate bounds
// this form).  Warp w owns the 16 x 32 sub-tile (16 (w & 3), 32 (w >> 2)) and
// sits out the products when that lies outside the tile; lane l accumulates
// rows 4 (l & 3) .. + 3 and columns 4 (l >> 2) .. + 3 of it with DFMA, reading
// its four A and four B values of a K-step as two 16-byte shared loads each.
__global__ void __launch_bounds__(256)
gemm_f64_kernel(BufTable bufs, const DevGemmOut* __restrict__ outs, const DevGemmSeg* __restrict__ segs,
                const DevGemmWork* __restrict__ work) {
    __shared__ __align__(16) double sA[GT_K][GT_LD];
    __shared__ __align__(16) double sB[GT_K][GT_LD];
    const DevGemmWork w = work[blockIdx.x];
    const DevGemmOut o = outs[w.out];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = 16 * (warp & 3) + 4 * (lane & 3);
    const int c0 = 32 * (warp >> 2) + 4 * (lane >> 2);
    const bool active = 16 * (warp & 3) < w.tm && 32 * (warp >> 2) < w.tn;
    double acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.0;
    for (int64_t s = o.s_begin; s < o.s_end; ++s) {
        const DevGemmSeg g = segs[s];
        const double* __restrict__ A = bufs.p[g.a_buf] + g.a_off;
        const double* __restrict__ B = bufs.p[g.b_buf] + g.b_off;
        const double alpha = g.alpha;
        for (int64_t k0 = 0; k0 < g.K; k0 += GT_K) {
            // A tile (GT_M x GT_K): element (m, k); rows past M read as zero
            for (int idx = threadIdx.x; idx < GT_M * GT_K; idx += 256) {
                int m, k;
                if (g.ta) { k = idx % GT_K; m = idx / GT_K; } else { m = idx % GT_M; k = idx / GT_M; }
                const int64_t gm = w.m0 + m, gk = k0 + k;
                double v = 0.0;
                if (m < w.tm && gm < o.M && gk < g.K) v = g.ta ? A[gk + gm * g.lda] : A[gm + gk * g.lda];
                sA[k][m] = v * alpha;
            }
            for (int idx = threadIdx.x; idx < GT_N * GT_K; idx += 256) {
                int n, k;
                if (g.tb) { n = idx % GT_N; k = idx / GT_N; } else { k = idx % GT_K; n = idx / GT_K; }
                const int64_t gn = w.n0 + n, gk = k0 + k;
                double v = 0.0;
                if (n < w.tn && gn < o.N && gk < g.K) v = g.tb ? B[gn + gk * g.ldb] : B[gk + gn * g.ldb];
                sB[k][n] = v;
            }
            __syncthreads();
            if (active) {
#pragma unroll
                for (int k = 0; k < GT_K; ++k) {
                    const double2 a01 = *(const double2*)&sA[k][r0];
                    const double2 a23 = *(const double2*)&sA[k][r0 + 2];
                    const double2 b01 = *(const double2*)&sB[k][c0];
                    const double2 b23 = *(const double2*)&sB[k][c0 + 2];
                    const double a[4] = {a01.x, a01.y, a23.x, a23.y};
                    const double b[4] = {b01.x, b01.y, b23.x, b23.y};
#pragma unroll
                    for (int i = 0; i < 4; ++i)
#pragma unroll
                        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
                }
            }
            __syncthreads();
        }
    }
    if (!active) return;
    double* __restrict__ C = bufs.p[o.c_buf] + o.c_off;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int64_t gn = w.n0 + c0 + j;
        if (c0 + j >= w.tn || gn >= o.N) continue;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int64_t gm = w.m0 + r0 + i;
            if (r0 + i < w.tm && gm < o.M) C[gm + gn * o.ldc] = acc[i][j];
        }
    }
}

// ------------------------------------------------------------------ plan upload / run
// Plan tables live in a memory pool of the library, one per device, and move through
// two non-blocking streams of its own: the upload stream (allocation and copy; the
// upload waits for this stream only, not for the caller's work) and the free stream
// (stream-ordered frees, after events recorded at the end of the plan's runs).
// cudaMalloc, cudaFree and cudaMemcpy each wait for the device or for the legacy
// stream; with them a host that plans the next site problem while the device runs
// the current boundary update waited for that update at every plan it dropped.
struct PlanMem {
    cudaMemPool_t pool = nullptr;
    cudaStream_t up = nullptr;
    cudaStream_t fr = nullptr;
};
static std::mutex g_pm_mu;
static PlanMem g_pm[64];
static thread_local const PlanMem* t_up = nullptr;  // the target of upload_vec while qcm_plan_upload runs

static int plan_mem(int dev, PlanMem** out) {
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return QCM_E_RANGE; }
    std::lock_guard<std::mutex> lk(g_pm_mu);
    PlanMem& m = g_pm[dev];
    if (!m.pool) {
        cudaMemPoolProps props = {};
        props.allocType = cudaMemAllocationTypePinned;
        props.handleTypes = cudaMemHandleTypeNone;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = dev;
        cudaMemPool_t pool;
        QCM_CUDA(cudaMemPoolCreate(&pool, &props));
        // keep up to 4 GiB of freed tables for the next plans instead of returning them to
        // the device at every synchronisation
        uint64_t keep = uint64_t(4) << 30;
        QCM_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
        if (!m.up) QCM_CUDA(cudaStreamCreateWithFlags(&m.up, cudaStreamNonBlocking));
        if (!m.fr) QCM_CUDA(cudaStreamCreateWithFlags(&m.fr, cudaStreamNonBlocking));
        m.pool = pool;
    }
    *out = &m;
    return QCM_OK;
}

static void free_stage_device(Stage& st, cudaStream_t fr) {
    for (void** d : {&st.d_a, &st.d_b, &st.d_c, &st.d_tcw, &st.d_cw, &st.d_ipanel, &st.d_ibuild, &st.d_iout,
                     &st.d_iseg, &st.d_iunit, &st.d_igather, &st.d_icoltab, &st.d_icimg, &st.d_cw_light,
                     &st.d_icost, &st.d_dterm, &st.d_dptr, &st.d_didx, &st.d_dw}) {
        if (*d) cudaFreeAsync(*d, fr);
        *d = nullptr;
    }
    st.n_cw = 0;
    st.n_cw_light = 0;
    if (st.ev_fork) cudaEventDestroy((cudaEvent_t)st.ev_fork);
    if (st.ev_join) cudaEventDestroy((cudaEvent_t)st.ev_join);
    if (st.side_stream) cudaStreamDestroy((cudaStream_t)st.side_stream);
    st.ev_fork = st.ev_join = st.side_stream = nullptr;
}

void release_plan_device(qcm_plan* p) {
    if (p->device < 0) return;
    int cur = -1;
    cudaGetDevice(&cur);
    if (cur != p->device) cudaSetDevice(p->device);
    PlanMem* pm = nullptr;
    if (plan_mem(p->device, &pm) == QCM_OK) {
        if (p->captured) {
            cudaDeviceSynchronize();
        } else {
            for (auto& se : p->run_ev) cudaStreamWaitEvent(pm->fr, (cudaEvent_t)se.second, 0);
            // copies of a failed upload may still be in flight on the upload stream
            cudaEvent_t e = nullptr;
            if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) == cudaSuccess) {
                cudaEventRecord(e, pm->up);
                cudaStreamWaitEvent(pm->fr, e, 0);
                cudaEventDestroy(e);
            }
        }
        for (auto& st : p->stages) free_stage_device(st, pm->fr);
    }
    for (auto& se : p->run_ev) cudaEventDestroy((cudaEvent_t)se.second);
    p->run_ev.clear();
    if (cur >= 0 && cur != p->device) cudaSetDevice(cur);
}

// pageable source: cudaMemcpyAsync has staged the bytes when it returns, so v may go
template <class T, class A>
static int upload_vec(const std::vector<T, A>& v, void** d) {
    if (!t_up) { set_error("plan tables uploaded outside qcm_plan_upload"); return QCM_E_STATE; }
    size_t bytes = std::max<size_t>(v.size(), 1) * sizeof(T);
    cudaError_t e = cudaMallocFromPoolAsync(d, bytes, t_up->pool, t_up->up);
    if (e != cudaSuccess) {
        *d = nullptr;
        set_error(std::string("cudaMallocFromPoolAsync: ") + cudaGetErrorString(e));
        return QCM_E_NOMEM;
    }
    if (!v.empty()) QCM_CUDA(cudaMemcpyAsync(*d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, t_up->up));
    return QCM_OK;
}

static int upload_images(Stage& st) {
    int rc = QCM_OK;
    if (st.img.units.empty()) return QCM_OK;
    if ((rc = upload_vec(st.img.panels, &st.d_ipanel))) return rc;
    if ((rc = upload_vec(st.img.build, &st.d_ibuild))) return rc;
    if ((rc = upload_vec(st.img.outs, &st.d_iout))) return rc;
    if ((rc = upload_vec(st.img.segs, &st.d_iseg))) return rc;
    if ((rc = upload_vec(st.img.units, &st.d_iunit))) return rc;
    if ((rc = upload_vec(st.img.gather, &st.d_igather))) return rc;
    if ((rc = upload_vec(st.img.coltab, &st.d_icoltab))) return rc;
    if ((rc = upload_vec(st.img.cimg, &st.d_icimg))) return rc;
    if (st.img.ares && (rc = upload_vec(st.img.cost, &st.d_icost))) return rc;
    return QCM_OK;
}

static int upload_stage(Stage& st) {
    int rc = QCM_OK;
    if (st.kind == ST_DOT) {
        std::vector<DevDotTerm> t(st.aterm.size());
        for (const AxpyOut& o : st.aout) {
            if (o.rows >= (int64_t(1) << 31) || o.cols >= (int64_t(1) << 31)) {
                set_error("dot tile too large");
                return QCM_E_RANGE;
            }
            for (int64_t k = o.t_begin; k < o.t_end; ++k) {
                const AxpyTerm& a = st.aterm[k];
                t[k] = {a.src_off, a.lds, o.dst_off, o.ldd, (int32_t)o.rows, (int32_t)o.cols, a.src_buf, o.dst_buf};
            }
        }
        // terms of each parameter in ascending term order (counting sort)
        std::vector<int64_t> ptr(st.n_tt + 1, 0), idx(st.dot_tt.size());
        for (int32_t tt : st.dot_tt) {
            if (tt < 0 || tt >= st.n_tt) { set_error("dot parameter index out of range"); return QCM_E_RANGE; }
            ++ptr[tt + 1];
        }
        for (int32_t i = 0; i < st.n_tt; ++i) ptr[i + 1] += ptr[i];
        std::vector<int64_t> fill(ptr.begin(), ptr.end() - 1);
        for (size_t k = 0; k < st.dot_tt.size(); ++k) idx[fill[st.dot_tt[k]]++] = (int64_t)k;
        if ((rc = upload_vec(t, &st.d_dterm))) return rc;
        if ((rc = upload_vec(ptr, &st.d_dptr))) return rc;
        if ((rc = upload_vec(idx, &st.d_didx))) return rc;
        if ((rc = upload_vec(st.dot_w, &st.d_dw))) return rc;
        st.n_work = (int64_t)t.size();
        return QCM_OK;
    }
    if (st.kind == ST_AXPY) {
        std::vector<DevAxpyOut> o(st.aout.size());
        std::vector<DevAxpyTerm> t(st.aterm.size());
        std::vector<DevAxpyWork> w;
        for (size_t i = 0; i < st.aout.size(); ++i) {
            const AxpyOut& a = st.aout[i];
            const int64_t pt = tile_pitch(st, a);
            o[i] = {a.dst_off, a.ldd, a.rows, a.cols, a.t_begin, a.t_end, a.dst_buf, (int32_t)(pt > 0 ? pt : 0)};
            // column chunks of at most ~8192 elements per work item
            int64_t cc = std::max<int64_t>(1, 8192 / std::max<int64_t>(1, a.rows));
            for (int64_t c0 = 0; c0 < a.cols; c0 += cc) w.push_back({(int64_t)i, c0, std::min(a.cols, c0 + cc)});
        }
        for (size_t i = 0; i < st.aterm.size(); ++i) {
            const AxpyTerm& a = st.aterm[i];
            t[i] = {a.src_off, a.lds, a.alpha, a.src_buf, 0};
        }
        if ((rc = upload_vec(o, &st.d_a))) return rc;
        if ((rc = upload_vec(t, &st.d_b))) return rc;
        if ((rc = upload_vec(w, &st.d_c))) return rc;
        st.n_work = (int64_t)w.size();
        st.src_buf = st.aterm.empty() ? -1 : st.aterm[0].src_buf;
        for (const AxpyTerm& a : st.aterm)
            if (a.src_buf != st.src_buf) { st.src_buf = -2; break; }
        std::vector<DevAxpyChunk> cw;
        if (st.src_buf >= 0 && build_chunk_work(st, cw) && !cw.empty() && cw.size() < 0x7fffffffULL) {
            if ((rc = upload_vec(cw, &st.d_cw))) return rc;
            st.n_cw = (int64_t)cw.size();
            if (!st.img.units.empty() && st.heavy.size() == st.aout.size()) {
                // the outputs the dense groups do not compute, in the same order
                std::vector<DevAxpyChunk> lw;
                for (const DevAxpyChunk& c : cw)
                    if (!st.heavy[c.out]) lw.push_back(c);
                if (!lw.empty() && (rc = upload_vec(lw, &st.d_cw_light))) return rc;
                st.n_cw_light = (int64_t)lw.size();
                if ((rc = upload_images(st))) return rc;
                // the dense groups' stream has the highest priority: whenever an SM frees
                // up, their CTAs are placed before more gather CTAs, so the two overlap
                cudaStream_t ss;
                cudaEvent_t e0, e1;
                int least = 0, greatest = 0;
                QCM_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
                QCM_CUDA(cudaStreamCreateWithPriority(&ss, cudaStreamNonBlocking, greatest));
                st.side_stream = ss;
                QCM_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
                st.ev_fork = e0;
                QCM_CUDA(cudaEventCreateWithFlags(&e1, cudaEventDisableTiming));
                st.ev_join = e1;
            }
        }
    } else if (st.kind == ST_GEMM) {
        std::vector<DevGemmOut> o(st.gout.size());
        std::vector<DevGemmSeg> s(st.gseg.size());
        std::vector<DevGemmWork> w;
        for (size_t i = 0; i < st.gout.size(); ++i) {
            const GemmOut& g = st.gout[i];
            o[i] = {g.c_off, g.ldc, g.M, g.N, g.s_begin, g.s_end, g.c_buf, 0};
            // tiles of at most 64 x 64, the last ones of a block cut to it (rows in steps of 16,
            // columns in steps of 32): the FP64 products spend little work on padding
            for (int64_t m0 = 0; m0 < g.M; m0 += GT_M) {
                const int32_t tm = (int32_t)std::min<int64_t>(GT_M, (g.M - m0 + 15) / 16 * 16);
                for (int64_t n0 = 0; n0 < g.N; n0 += GT_N) {
                    const int32_t tn = (int32_t)std::min<int64_t>(GT_N, (g.N - n0 + 31) / 32 * 32);
                    w.push_back({(int64_t)i, m0, n0, tm, tn});
                }
            }
        }
        for (size_t i = 0; i < st.gseg.size(); ++i) {
            const GemmSeg& g = st.gseg[i];
            s[i] = {g.a_off, g.lda, g.b_off, g.ldb, g.K, g.alpha, g.a_buf, g.ta, g.b_buf, g.tb};
        }
        if ((rc = upload_vec(o, &st.d_a))) return rc;
        if ((rc = upload_vec(s, &st.d_b))) return rc;
        if ((rc = upload_vec(w, &st.d_c))) return rc;
        st.n_work = (int64_t)w.size();
        std::vector<int64_t> tw;
        tc_build_work(st, tw);
        if ((rc = upload_vec(tw, &st.d_tcw))) return rc;
        st.n_tcw = (int64_t)tw.size() / 3;
        if ((rc = upload_images(st))) return rc;
    }
    return QCM_OK;
}

// The image-executor forms: BF16x3 (6 slice products per K-step) and BF16x2 (3).
static inline bool img_form(int precision) {
    return precision == QCM_PREC_BF16X3 || precision == QCM_PREC_BF16X2;
}
static inline int img_products(int precision) { return precision == QCM_PREC_BF16X2 ? 3 : 6; }

static int launch_axpy(const Stage& st, const BufTable& bt, int precision, cudaStream_t s) {
    if (st.n_work == 0) return QCM_OK;
    if (st.n_work > 0x7fffffffLL) { set_error("axpy work list too large"); return QCM_E_RANGE; }
    const auto* O = (const DevAxpyOut*)st.d_a;
    const auto* T = (const DevAxpyTerm*)st.d_b;
    const auto* W = (const DevAxpyWork*)st.d_c;
    const unsigned g = (unsigned)st.n_work;
    // FP64 form: the column-chunk executor (it is FP64-FMA bound either way and
    // measured faster); mixed forms: the contiguous-chunk executor.
    if (st.src_buf >= 0 && st.n_cw > 0 && precision != QCM_PREC_FP64) {
        const bool src32 = (bt.f32mask >> st.src_buf) & 1u;
        const auto* CW = (const DevAxpyChunk*)st.d_cw;
        unsigned gc = (unsigned)st.n_cw;
        if (img_form(precision) && bt.p[QCM_BUF_IMG] && st.d_iunit) {
            // BF16x3 / BF16x2 with images: the dense groups on the tensor cores on the stage's
            // high-priority side stream, and the gather of the other outputs on the caller's
            // stream, the side stream forked from and joined back into it (disjoint outputs)
            cudaStream_t ss = (cudaStream_t)st.side_stream;
            const bool fork = ss && st.n_cw_light > 0;
            if (fork) {
                QCM_CUDA(cudaEventRecord((cudaEvent_t)st.ev_fork, s));
                QCM_CUDA(cudaStreamWaitEvent(ss, (cudaEvent_t)st.ev_fork, 0));
                const int rc = tc_img_launch(st, bt.p, bt.f32mask, (void*)ss, img_products(precision));
                const auto* LW = (const DevAxpyChunk*)st.d_cw_light;
                const unsigned gl = (unsigned)st.n_cw_light;
                if (src32) gather_axpy_contig<float, float><<<gl, CG_THREADS, 0, s>>>(bt, O, T, LW);
                else gather_axpy_contig<float, double><<<gl, CG_THREADS, 0, s>>>(bt, O, T, LW);
                const cudaError_t le = cudaGetLastError();
                // join even after a failed launch, so that no work is left forked
                QCM_CUDA(cudaEventRecord((cudaEvent_t)st.ev_join, ss));
                QCM_CUDA(cudaStreamWaitEvent(s, (cudaEvent_t)st.ev_join, 0));
                if (rc) return rc;
                if (le != cudaSuccess) { set_error(std::string("gather launch: ") + cudaGetErrorString(le)); return QCM_E_CUDA; }
                return QCM_OK;
            }
            int rc = tc_img_launch(st, bt.p, bt.f32mask, (void*)s, img_products(precision));
            if (rc) return rc;
            CW = (const DevAxpyChunk*)st.d_cw_light;
            gc = (unsigned)st.n_cw_light;
            if (gc == 0) return QCM_OK;
        }
        if (src32) {
            gather_axpy_contig<float, float><<<gc, CG_THREADS, 0, s>>>(bt, O, T, CW);
        } else {
            gather_axpy_contig<float, double><<<gc, CG_THREADS, 0, s>>>(bt, O, T, CW);
        }
    } else if (st.src_buf >= 0) {
        const bool src32 = (bt.f32mask >> st.src_buf) & 1u;
        if (precision == QCM_PREC_FP64) {
            if (src32) { set_error("the FP64 form takes FP64 buffers only"); return QCM_E_INVALID; }
            gather_axpy_uniform<double, double><<<g, AXPY_THREADS, 0, s>>>(bt, O, T, W);
        } else if (src32) {
            gather_axpy_uniform<float, float><<<g, AXPY_THREADS, 0, s>>>(bt, O, T, W);
        } else {
            gather_axpy_uniform<float, double><<<g, AXPY_THREADS, 0, s>>>(bt, O, T, W);
        }
    } else if (precision == QCM_PREC_FP64) {
        gather_axpy_kernel<double><<<g, AXPY_THREADS, 0, s>>>(bt, O, T, W);
    } else {
        gather_axpy_kernel<float><<<g, AXPY_THREADS, 0, s>>>(bt, O, T, W);
    }
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

static int launch_gemm(const Stage& st, const BufTable& bt, int precision, cudaStream_t s) {
    if (st.n_work == 0) return QCM_OK;
    if (st.n_work > 0x7fffffffLL) { set_error("gemm work list too large"); return QCM_E_RANGE; }
    if (img_form(precision) && bt.p[QCM_BUF_IMG] && st.d_iunit)
        return tc_img_launch(st, bt.p, bt.f32mask, (void*)s, img_products(precision));
    if (precision == QCM_PREC_BF16X2) {
        set_error("the BF16x2 form runs on the image executor only: pass the operand-image slot");
        return QCM_E_INVALID;
    }
    if (precision != QCM_PREC_FP64)
        return tc_launch(st.d_a, st.d_b, st.d_tcw, st.n_tcw, bt.p, bt.f32mask, precision, (void*)s);
    if (bt.f32mask) { set_error("the FP64 form takes FP64 buffers only"); return QCM_E_INVALID; }
    gemm_f64_kernel<<<(unsigned)st.n_work, 256, 0, s>>>(bt, (const DevGemmOut*)st.d_a, (const DevGemmSeg*)st.d_b,
                                                         (const DevGemmWork*)st.d_c);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

// Kernels one stage launches on the path launch_axpy / launch_gemm take.
static int stage_kernels(const Stage& st, const BufTable& bt, int precision) {
    const bool images = img_form(precision) && bt.p[QCM_BUF_IMG] && st.d_iunit;
    if (st.kind == ST_AXPY) {
        if (st.n_work == 0) return 0;
        if (images && st.src_buf >= 0 && st.n_cw > 0)
            return (st.n_cw_light > 0 ? 1 : 0) + (st.img.build.empty() ? 0 : 1) + 1;
        return 1;
    }
    if (st.kind == ST_GEMM) {
        if (st.n_work == 0) return 0;
        return images ? (st.img.build.empty() ? 0 : 1) + 1 : 1;
    }
    if (st.kind == ST_DOT) return (st.n_work > 0 ? 1 : 0) + (st.n_tt > 0 ? 1 : 0);
    return 0;
}

static int launch_dot(const Stage& st, const BufTable& bt, cudaStream_t s) {
    double* g = bt.p[st.dot_buf];
    double* out = bt.p[QCM_BUF_OUT];
    if (!out || (st.n_work > 0 && !g)) { set_error("missing buffer for the gradient stage"); return QCM_E_INVALID; }
    if (st.n_work > 0) {
        const unsigned grid = (unsigned)std::min<int64_t>(st.n_work, 152 * 16);
        dot_terms_kernel<<<grid, DOT_THREADS, 0, s>>>(bt, (const DevDotTerm*)st.d_dterm, st.n_work, g);
        QCM_CUDA(cudaGetLastError());
    }
    if (st.n_tt > 0) {
        dot_reduce_kernel<<<(st.n_tt + 127) / 128, 128, 0, s>>>((const int64_t*)st.d_dptr, (const int64_t*)st.d_didx,
                                                              (const double*)st.d_dw, g, st.n_tt, out);
        QCM_CUDA(cudaGetLastError());
    }
    return QCM_OK;
}

// ------------------------------------------------------------------ vector kernels
constexpr int RED_THREADS = 256;
constexpr int RED_BLOCKS = 304;  // 2 x 152 SMs

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ double block_sum(double v) {
    __shared__ double ws[RED_THREADS / 32];
    v = warp_sum(v);
    const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
    __syncthreads();
    if (lane == 0) ws[wid] = v;
    __syncthreads();
    double r = 0.0;
    if (wid == 0) {
        r = (lane < RED_THREADS / 32) ? ws[lane] : 0.0;
        r = warp_sum(r);
    }
    return r;  // valid in thread 0
}

__global__ void __launch_bounds__(RED_THREADS)
multi_dot_partial(const double* const* __restrict__ v, int nvec, const double* __restrict__ y, int64_t n,
                  double* __restrict__ partial) {
    // partial[k * gridDim.x + blockIdx.x]
    for (int k = 0; k < nvec; ++k) {
        const double* __restrict__ x = v[k];
        double s = 0.0;
        for (int64_t i = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RED_THREADS)
            s = fma(x[i], y[i], s);
        s = block_sum(s);
        if (threadIdx.x == 0) partial[(int64_t)k * gridDim.x + blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(RED_THREADS)
multi_dot_final(const double* __restrict__ partial, int nparts, int nvec, double* __restrict__ out, int do_sqrt) {
    for (int k = 0; k < nvec; ++k) {
        double s = 0.0;
        for (int i = threadIdx.x; i < nparts; i += RED_THREADS) s += partial[(int64_t)k * nparts + i];
        s = block_sum(s);
        if (threadIdx.x == 0) out[k] = do_sqrt ? sqrt(s) : s;
    }
}

__global__ void axpby_kernel(double a, const double* __restrict__ x, double b, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
        y[i] = (b == 0.0) ? a * x[i] : fma(a, x[i], b * y[i]);
}

constexpr int LIN_MAX = 32;
struct LinArgs { const double* x[LIN_MAX]; double c[LIN_MAX]; int n; };

__global__ void lincomb_kernel(LinArgs args, double* __restrict__ y, int64_t n) {
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < args.n; ++k) s = fma(args.c[k], args.x[k][i], s);
        y[i] = s;
    }
}

// ------------------------------------------------------------------ allocation-free multi-dot
// Scratch of qcm_multi_dot_noalloc: one partial sum per (vector, block).  It is
// a file-scope device array, so every GPU that loads this library holds it
// (NOALLOC_MAX_VEC * RED_BLOCKS doubles = 76 KiB) until the process exits.
constexpr int NOALLOC_MAX_VEC = 32;
static __device__ __align__(256) double g_noalloc_partial[NOALLOC_MAX_VEC * RED_BLOCKS];

struct DotPtrs { const double* x[NOALLOC_MAX_VEC]; };

// Same reduction as multi_dot_partial, with the vector pointers passed by value
// instead of through a device-side pointer table.
__global__ void __launch_bounds__(RED_THREADS)
multi_dot_partial_byval(DotPtrs v, int nvec, const double* __restrict__ y, int64_t n, double* __restrict__ partial) {
    for (int k = 0; k < nvec; ++k) {
        const double* __restrict__ x = v.x[k];
        double s = 0.0;
        for (int64_t i = (int64_t)blockIdx.x * RED_THREADS + threadIdx.x; i < n; i += (int64_t)gridDim.x * RED_THREADS)
            s = fma(x[i], y[i], s);
        s = block_sum(s);
        if (threadIdx.x == 0) partial[(int64_t)k * gridDim.x + blockIdx.x] = s;
    }
}

// Segmented dots for batched eigensolvers: out[j * nseg + k] = sum over segment k
// ([seg[k], seg[k+1]) of the concatenated vectors) of V_j[i] * y[i]; one block per
// (segment, vector), fixed reduction order.
__global__ void __launch_bounds__(RED_THREADS)
seg_multi_dot_kernel(DotPtrs v, const double* __restrict__ y, const int64_t* __restrict__ seg, int nseg,
                     double* __restrict__ out) {
    const int k = blockIdx.x, j = blockIdx.y;
    const double* __restrict__ x = v.x[j];
    const int64_t e = seg[k + 1];
    double s = 0.0;
    for (int64_t i = seg[k] + threadIdx.x; i < e; i += RED_THREADS) s = fma(x[i], y[i], s);
    s = block_sum(s);
    if (threadIdx.x == 0) out[(int64_t)j * nseg + k] = s;
}

// Device address of g_noalloc_partial per device, looked up once (set-up of the
// first call on that device).
static std::mutex g_noalloc_mu;
static double* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(double** out) {
    int dev = 0;
    QCM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return QCM_E_RANGE; }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partial);
        if (e != cudaSuccess || !p) {
            set_error(std::string("cudaGetSymbolAddress(g_noalloc_partial): ") + cudaGetErrorString(e));
            return QCM_E_CUDA;
        }
        g_noalloc_ptr[dev] = (double*)p;
    }
    *out = g_noalloc_ptr[dev];
    return QCM_OK;
}

// per-device reduction workspace owned by the library (allocated on first use)
struct RedWs { double* partial = nullptr; const double** ptrs = nullptr; };
static std::mutex g_ws_mu;
static RedWs g_ws[64];

static int get_ws(RedWs** ws) {
    int dev = 0;
    QCM_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) { set_error("device ordinal out of range"); return QCM_E_RANGE; }
    std::lock_guard<std::mutex> lk(g_ws_mu);
    RedWs& w = g_ws[dev];
    if (!w.partial) {
        if (cudaMalloc(&w.partial, sizeof(double) * RED_BLOCKS * LIN_MAX) != cudaSuccess) {
            set_error("cudaMalloc of the reduction workspace failed");
            return QCM_E_NOMEM;
        }
        if (cudaMalloc((void**)&w.ptrs, sizeof(double*) * LIN_MAX) != cudaSuccess) {
            set_error("cudaMalloc of the pointer table failed");
            return QCM_E_NOMEM;
        }
    }
    *ws = &w;
    return QCM_OK;
}

}  // namespace qcm

using namespace qcm;

extern "C" {

int qcm_plan_upload(qcm_plan* p) {
    if (!p) { set_error("null plan"); return QCM_E_INVALID; }
    if (p->uploaded) return QCM_OK;
    int dev = 0;
    QCM_CUDA(cudaGetDevice(&dev));
    PlanMem* pm = nullptr;
    int rc = plan_mem(dev, &pm);
    if (rc) return rc;
    p->device = dev;  // what a failed upload left is freed on this device
    t_up = pm;
    for (auto& st : p->stages) {
        rc = upload_stage(st);
        if (rc) break;
    }
    t_up = nullptr;
    if (rc) return rc;
    // the tables are on the device when the upload returns (a wait for the upload
    // stream alone), so runs need no ordering against it, captured runs included
    QCM_CUDA(cudaStreamSynchronize(pm->up));
    p->uploaded = true;
    return QCM_OK;
}

int qcm_plan_run(qcm_plan* p, double* const* bufs, int32_t precision, void* stream) {
    return qcm_plan_run_stages(p, bufs, precision, stream, 0, -1);
}

int qcm_plan_run_stages(qcm_plan* p, double* const* bufs, int32_t precision, void* stream, int32_t first,
                        int32_t last) {
    // FP64 form: every slot FP64.  Mixed forms: scratch slots FP32, caller slots FP64.
    uint32_t mask = (precision == QCM_PREC_FP64) ? 0u
                                                 : ((1u << QCM_BUF_S0) | (1u << QCM_BUF_S1) | (1u << QCM_BUF_S2));
    return qcm_plan_run_typed(p, bufs, mask, precision, stream, first, last);
}

int qcm_plan_run_typed(qcm_plan* p, double* const* bufs, uint32_t f32mask, int32_t precision, void* stream,
                       int32_t first, int32_t last) {
    if (!p || !bufs) { set_error("null argument"); return QCM_E_INVALID; }
    if (last < 0 || last >= (int32_t)p->stages.size()) last = (int32_t)p->stages.size() - 1;
    if (first < 0) first = 0;
    if (!p->uploaded) { set_error("plan not uploaded"); return QCM_E_STATE; }
    int dev = 0;
    QCM_CUDA(cudaGetDevice(&dev));
    if (dev != p->device) { set_error("plan was uploaded to another device"); return QCM_E_STATE; }
    if (precision != QCM_PREC_FP64 && precision != QCM_PREC_TF32 && precision != QCM_PREC_BF16X3 &&
        precision != QCM_PREC_BF16X2) {
        set_error("unknown precision");
        return QCM_E_INVALID;
    }
    if ((p->kind == PK_GRAD || p->kind == PK_DIAG) && (precision != QCM_PREC_FP64 || f32mask != 0)) {
        set_error(p->kind == PK_GRAD ? "energy-gradient plans run in the FP64 form only"
                                     : "diagonal plans run in the FP64 form only");
        return QCM_E_INVALID;
    }
    BufTable bt;
    for (int i = 0; i < QCM_NBUF; ++i) bt.p[i] = bufs[i];
    bt.f32mask = f32mask;
    cudaStream_t s = (cudaStream_t)stream;
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    QCM_CUDA(cudaStreamIsCapturing(s, &cap));
    // a graph keeps reading the tables after the capture: such a plan's teardown
    // waits for the device instead of for events of its runs
    if (cap != cudaStreamCaptureStatusNone) p->captured = true;
    p->last_kernels = 0;
    for (int32_t si = first; si <= last; ++si) {
        Stage& st = p->stages[si];
        int rc = QCM_OK;
        p->last_kernels += stage_kernels(st, bt, precision);
        if (st.kind == ST_ZERO) {
            if (st.zlen > 0) {
                if (!bufs[st.zbuf]) { set_error("missing scratch buffer"); return QCM_E_INVALID; }
                const size_t esz = ((f32mask >> st.zbuf) & 1u) ? sizeof(float) : sizeof(double);
                QCM_CUDA(cudaMemsetAsync(bufs[st.zbuf], 0, esz * st.zlen, s));
            }
        } else if (st.kind == ST_AXPY) {
            rc = launch_axpy(st, bt, precision, s);
        } else if (st.kind == ST_DOT) {
            rc = launch_dot(st, bt, s);
        } else {
            rc = launch_gemm(st, bt, precision, s);
        }
        if (rc) return rc;
    }
    if (cap == cudaStreamCaptureStatusNone) {
        cudaEvent_t ev = nullptr;
        for (auto& se : p->run_ev)
            if (se.first == (void*)s) { ev = (cudaEvent_t)se.second; break; }
        if (!ev) {
            QCM_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
            p->run_ev.push_back({(void*)s, (void*)ev});
        }
        QCM_CUDA(cudaEventRecord(ev, s));
    }
    return QCM_OK;
}

int qcm_multi_dot(const double* const* v, int32_t nvec, const double* y, int64_t n, double* out, void* stream) {
    if (nvec < 0 || nvec > LIN_MAX) { set_error("qcm_multi_dot: nvec out of range"); return QCM_E_RANGE; }
    if (nvec == 0) return QCM_OK;
    RedWs* ws = nullptr;
    int rc = get_ws(&ws);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    QCM_CUDA(cudaMemcpyAsync(ws->ptrs, v, sizeof(double*) * nvec, cudaMemcpyHostToDevice, s));
    multi_dot_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(ws->ptrs, nvec, y, n, ws->partial);
    QCM_CUDA(cudaGetLastError());
    multi_dot_final<<<1, RED_THREADS, 0, s>>>(ws->partial, RED_BLOCKS, nvec, out, 0);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

int qcm_seg_multi_dot(const double* const* v, int32_t nvec, const double* y, const int64_t* seg_off, int32_t nseg,
                      double* out, void* stream) {
    if (nvec < 0 || nvec > NOALLOC_MAX_VEC) {
        set_error("qcm_seg_multi_dot: nvec " + std::to_string(nvec) + " out of range (at most " +
                  std::to_string(NOALLOC_MAX_VEC) + ")");
        return QCM_E_RANGE;
    }
    if (nseg < 0 || nseg > 65535) { set_error("qcm_seg_multi_dot: nseg out of range"); return QCM_E_RANGE; }
    if (nvec == 0 || nseg == 0) return QCM_OK;
    if (!v || !y || !seg_off || !out) { set_error("qcm_seg_multi_dot: null pointer"); return QCM_E_INVALID; }
    DotPtrs args;
    for (int k = 0; k < NOALLOC_MAX_VEC; ++k) args.x[k] = (k < nvec) ? v[k] : nullptr;
    for (int k = 0; k < nvec; ++k)
        if (!args.x[k]) { set_error("qcm_seg_multi_dot: null vector pointer"); return QCM_E_INVALID; }
    seg_multi_dot_kernel<<<dim3((unsigned)nseg, (unsigned)nvec), RED_THREADS, 0, (cudaStream_t)stream>>>(
        args, y, seg_off, nseg, out);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

int qcm_multi_dot_noalloc(const double* const* v, int32_t nvec, const double* y, int64_t n, double* out,
                          void* stream) {
    if (nvec < 0 || nvec > NOALLOC_MAX_VEC) {
        set_error("qcm_multi_dot_noalloc: nvec " + std::to_string(nvec) + " exceeds the fixed scratch capacity of " +
                  std::to_string(NOALLOC_MAX_VEC) + " vectors");
        return QCM_E_RANGE;
    }
    if (n < 0) { set_error("qcm_multi_dot_noalloc: negative length"); return QCM_E_INVALID; }
    if (nvec == 0) return QCM_OK;
    if (!v || !y || !out) { set_error("qcm_multi_dot_noalloc: null pointer"); return QCM_E_INVALID; }
    double* partial = nullptr;
    int rc = noalloc_scratch(&partial);
    if (rc) return rc;
    DotPtrs args;
    for (int k = 0; k < NOALLOC_MAX_VEC; ++k) args.x[k] = (k < nvec) ? v[k] : nullptr;
    for (int k = 0; k < nvec; ++k)
        if (!args.x[k]) { set_error("qcm_multi_dot_noalloc: null vector pointer"); return QCM_E_INVALID; }
    cudaStream_t s = (cudaStream_t)stream;
    // every partial read by multi_dot_final is written by this launch first: nothing to clear
    multi_dot_partial_byval<<<RED_BLOCKS, RED_THREADS, 0, s>>>(args, nvec, y, n, partial);
    QCM_CUDA(cudaGetLastError());
    multi_dot_final<<<1, RED_THREADS, 0, s>>>(partial, RED_BLOCKS, nvec, out, 0);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

int qcm_dot(const double* x, const double* y, int64_t n, double* out, void* stream) {
    const double* v[1] = {x};
    return qcm_multi_dot(v, 1, y, n, out, stream);
}

int qcm_nrm2(const double* x, int64_t n, double* out, void* stream) {
    RedWs* ws = nullptr;
    int rc = get_ws(&ws);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const double* v[1] = {x};
    QCM_CUDA(cudaMemcpyAsync(ws->ptrs, v, sizeof(double*), cudaMemcpyHostToDevice, s));
    multi_dot_partial<<<RED_BLOCKS, RED_THREADS, 0, s>>>(ws->ptrs, 1, x, n, ws->partial);
    QCM_CUDA(cudaGetLastError());
    multi_dot_final<<<1, RED_THREADS, 0, s>>>(ws->partial, RED_BLOCKS, 1, out, 1);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

int qcm_axpby(double a, const double* x, double b, double* y, int64_t n, void* stream) {
    if (n <= 0) return QCM_OK;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    axpby_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(a, x, b, y, n);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

int qcm_lincomb(const double* const* x, const double* coef, int32_t nvec, double* y, int64_t n, void* stream) {
    if (nvec < 1 || nvec > LIN_MAX) { set_error("qcm_lincomb: nvec out of range"); return QCM_E_RANGE; }
    LinArgs args;
    for (int k = 0; k < nvec; ++k) { args.x[k] = x[k]; args.c[k] = coef[k]; }
    args.n = nvec;
    int blocks = (int)std::min<int64_t>((n + 255) / 256, 152 * 8);
    if (blocks < 1) return QCM_OK;
    lincomb_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(args, y, n);
    QCM_CUDA(cudaGetLastError());
    return QCM_OK;
}

}  // extern "C"
