// Tensor-core (tcgen05 / TMEM) grouped block products for the mixed-precision
// sigma vector on sm_103a.
//
// Same work list as the FP64 executor: every CTA owns one 128 x 64 output tile
// of one output block and accumulates all of its segments (the split-K over
// MPO bond indices) in a TMEM accumulator (FP32), then writes the tile once in
// FP64.  Operands are FP64 in HBM; each K-chunk is loaded, scaled, split into
// low-precision slices and stored in shared memory in the canonical K-major
// "no swizzle" UMMA layout (8-row x 16-byte core matrices), from where one
// elected thread issues tcgen05.mma:
//   PREC_TF32   : 1 slice, kind::tf32 (round-to-nearest TF32), 1 product;
//   PREC_BF16X3 : 3 BF16 slices a = a0+a1+a2, 6 products a_i b_j with i+j <= 2.
// FP32 accumulation in TMEM; completion through tcgen05.commit on an mbarrier.
// Every wait is bounded: on timeout the kernel records an error code in
// g_tc_status, still releases its TMEM and returns.
#include <cuda_runtime.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cstdint>
#include <string>

#include "plan.hpp"

namespace qcm {

constexpr int TC_BM = 128;      // MMA M (one TMEM lane per row)
constexpr int TC_BN = 64;       // MMA N (64 FP32 TMEM columns)
constexpr int TC_KB = 64;       // bytes of K per shared-memory chunk (4 core-matrix columns)
constexpr int TC_THREADS = 256;
constexpr unsigned TC_SPIN_LIMIT = 1u << 26;

__device__ int g_tc_status = 0;

struct TcOut { int64_t c_off, ldc, M, N, s_begin, s_end; int32_t c_buf, pad; };
struct TcSeg { int64_t a_off, lda, b_off, ldb, K; double alpha; int32_t a_buf, ta, b_buf, tb; };
struct TcWork { int64_t out, m0, n0; };
struct TcBufs { double* p[QCM_NBUF]; uint32_t f32mask; };

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// UMMA shared-memory matrix descriptor, K-major, no swizzle (layout type 0), version 1.
__device__ __forceinline__ uint64_t make_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    return d;
}

// Instruction descriptor: D=F32, A/B format, K-major A and B, N>>3, M>>4.
__host__ __device__ constexpr uint32_t make_idesc(uint32_t ab_format, int M, int N) {
    return (1u << 4) | (ab_format << 7) | (ab_format << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// byte offset of element (r, k) of a K-major tile whose rows hold TC_KB bytes, element size E
template <int E>
__device__ __forceinline__ uint32_t kmajor_off(int r, int k) {
    constexpr int T = 16 / E;                 // elements per 16-byte core row
    constexpr int CPR = TC_KB / 16;           // core-matrix columns per chunk
    return (uint32_t)((((r >> 3) * CPR) + (k / T)) * 128 + (r & 7) * 16 + (k % T) * E);
}

__device__ __forceinline__ uint32_t to_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return r;
}

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t phase) {
    for (unsigned it = 0; it < TC_SPIN_LIMIT; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done) : "r"(mbar), "r"(phase) : "memory");
        if (done) return true;
    }
    return false;
}

template <int PREC>
struct TcCfg;
template <>
struct TcCfg<QCM_PREC_TF32> {
    static constexpr int E = 4, SLICES = 1, NPROD = 1, KSTEP = 8;
    static constexpr uint32_t FMT = 2;  // TF32
};
template <>
struct TcCfg<QCM_PREC_BF16X3> {
    static constexpr int E = 2, SLICES = 3, NPROD = 6, KSTEP = 16;
    static constexpr uint32_t FMT = 1;  // BF16
};

// Split T = 16/E consecutive-K operand values into the MMA format and store
// them as one 16-byte vector per slice at byte offset `off` of slice 0 (further
// slices follow at `slice_bytes` strides).  All splitting arithmetic is FP32:
// the FP64 pipe of this part is far narrower than the FP32 one, and three BF16
// slices carry the 24 bits an FP32 value has.
template <int PREC>
__device__ __forceinline__ void put_vec(uint8_t* base, uint32_t off, uint32_t slice_bytes, const float* v,
                                        int nsl = 3) {
    if constexpr (PREC == QCM_PREC_TF32) {
        uint4 q;
        q.x = to_tf32(v[0]); q.y = to_tf32(v[1]); q.z = to_tf32(v[2]); q.w = to_tf32(v[3]);
        *reinterpret_cast<uint4*>(base + off) = q;
    } else {
        // pairs of values are rounded together (one packed bf16x2 conversion);
        // each slice takes the round-to-nearest BF16 of what the previous ones left
        uint32_t s0[4], s1[4], s2[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const float2 x = make_float2(v[2 * i], v[2 * i + 1]);
            const __nv_bfloat162 h0 = __float22bfloat162_rn(x);
            const float2 f0 = __bfloat1622float2(h0);
            const float2 r1 = make_float2(x.x - f0.x, x.y - f0.y);
            const __nv_bfloat162 h1 = __float22bfloat162_rn(r1);
            const float2 f1 = __bfloat1622float2(h1);
            const float2 r2 = make_float2(r1.x - f1.x, r1.y - f1.y);
            const __nv_bfloat162 h2 = __float22bfloat162_rn(r2);
            s0[i] = *reinterpret_cast<const uint32_t*>(&h0);
            s1[i] = *reinterpret_cast<const uint32_t*>(&h1);
            s2[i] = *reinterpret_cast<const uint32_t*>(&h2);
        }
        *reinterpret_cast<uint4*>(base + off) = make_uint4(s0[0], s0[1], s0[2], s0[3]);
        *reinterpret_cast<uint4*>(base + slice_bytes + off) = make_uint4(s1[0], s1[1], s1[2], s1[3]);
        if (nsl > 2)   // the BF16x2 form reads slices 0 and 1 only
            *reinterpret_cast<uint4*>(base + 2 * slice_bytes + off) = make_uint4(s2[0], s2[1], s2[2], s2[3]);
    }
}

// Load a K-chunk of one operand into shared memory.  Rows R (the M or N extent of
// the tile), KC elements of K; each work unit is T consecutive K of one row,
// written as one 16-byte vector.  `tr` selects the global storage order:
// tr == 0: element (r, k) at P[r + k*ld] (rows contiguous -> warps span rows);
// tr == 1: element (r, k) at P[k + r*ld] (K contiguous -> warps span K first).
template <int PREC, int R, int KC, int T>
__device__ __forceinline__ void load_chunk(uint8_t* sbase, uint32_t slice_bytes, const double* P64, const float* P32,
                                           bool f32, int tr, int64_t ld, int64_t r0, int64_t rlim, int64_t k0,
                                           int64_t klim, float scale) {
    constexpr int E = 16 / T;
    constexpr int KV = KC / T;  // vectors per row
    for (int u = threadIdx.x; u < R * KV; u += TC_THREADS) {
        int r, kv;
        if (tr) { kv = u % KV; r = u / KV; } else { r = u % R; kv = u / R; }
        // in-block offsets fit in 32 bits (the plan builder keeps blocks below 2^31 elements)
        const int gr = (int)(r0 + r);
        const int ld32 = (int)ld;
        float v[T];
#pragma unroll
        for (int j = 0; j < T; ++j) {
            const int gk = (int)(k0 + kv * T + j);
            float x = 0.0f;
            if (gr < rlim && gk < klim) {
                const int ix = tr ? gk + gr * ld32 : gr + gk * ld32;
                x = f32 ? __ldg(P32 + ix) : (float)__ldg(P64 + ix);
            }
            v[j] = scale * x;
        }
        put_vec<PREC>(sbase, kmajor_off<E>(r, kv * T), slice_bytes, v);
    }
}

template <int PREC>
__global__ void __launch_bounds__(TC_THREADS)
tc_gemm_kernel(TcBufs bufs, const TcOut* __restrict__ outs, const TcSeg* __restrict__ segs,
               const TcWork* __restrict__ work) {
    using Cfg = TcCfg<PREC>;
    constexpr int E = Cfg::E;
    constexpr int KC = TC_KB / E;                       // elements of K per chunk
    constexpr uint32_t A_BYTES = TC_BM * TC_KB;         // one slice of the A tile
    constexpr uint32_t B_BYTES = TC_BN * TC_KB;
    constexpr uint32_t STAGE_BYTES = Cfg::SLICES * (A_BYTES + B_BYTES);
    constexpr uint32_t LBO = 128;                       // next core matrix along K
    constexpr uint32_t SBO = (TC_KB / 16) * 128;        // next 8-row group
    constexpr uint32_t IDESC = make_idesc(Cfg::FMT, TC_BM, TC_BN);
    constexpr int NSTAGE = 2;

    extern __shared__ __align__(1024) uint8_t smem[];
    __shared__ __align__(8) uint64_t mbar[NSTAGE];
    __shared__ uint32_t tmem_base_sh;

    const int tid = threadIdx.x;
    const int warp = tid / 32, lane = tid % 32;
    const int quad = warp & 3;      // TMEM lanes 32*quad .. 32*quad+31 (tile rows)
    const int chalf = warp >> 2;    // tile columns 32*chalf .. 32*chalf+31
    const TcWork w = work[blockIdx.x];
    const TcOut o = outs[w.out];

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_base_sh)), "r"((uint32_t)TC_BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 0) {
        for (int i = 0; i < NSTAGE; ++i) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&mbar[i])));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_base_sh;
    const uint32_t trow = tmem + ((uint32_t)(quad * 32) << 16) + (uint32_t)(chalf * 32);

    uint32_t phase[NSTAGE] = {0u, 0u};
    bool pending[NSTAGE] = {false, false};
    bool aborted = false;
    // Accumulators of this thread's row and 32 columns: each segment (one block
    // product of the split-K sum) accumulates in FP32 in TMEM, then is drained
    // into these with a compensated (two-sum) FP32 addition.
    float acc_hi[32], acc_lo[32];  // compensated (two-sum) FP32 accumulation across segments
#pragma unroll
    for (int j = 0; j < 32; ++j) { acc_hi[j] = 0.0f; acc_lo[j] = 0.0f; }
    int chunk = 0;

    for (int64_t s = o.s_begin; s < o.s_end && !aborted; ++s) {
        const TcSeg g = segs[s];
        if (g.K <= 0) continue;
        const bool a32 = (bufs.f32mask >> g.a_buf) & 1u, b32 = (bufs.f32mask >> g.b_buf) & 1u;
        const double* __restrict__ A = bufs.p[g.a_buf] + (a32 ? 0 : g.a_off);
        const double* __restrict__ B = bufs.p[g.b_buf] + (b32 ? 0 : g.b_off);
        const float* __restrict__ Af = (const float*)bufs.p[g.a_buf] + (a32 ? g.a_off : 0);
        const float* __restrict__ Bf = (const float*)bufs.p[g.b_buf] + (b32 ? g.b_off : 0);
        const float alpha = (float)g.alpha;
        bool first = true;  // the first MMA of a segment overwrites the accumulator
        for (int64_t k0 = 0; k0 < g.K; k0 += KC) {
            const int st = chunk & 1;
            uint8_t* sA = smem + st * STAGE_BYTES;
            uint8_t* sB = sA + Cfg::SLICES * A_BYTES;
            // the MMAs that last read this stage must have finished before it is overwritten
            if (pending[st]) {
                int to = mbar_wait(smem_u32(&mbar[st]), phase[st]) ? 0 : 1;
                phase[st] ^= 1u;
                pending[st] = false;
                if (__syncthreads_or(to)) { aborted = true; break; }
            }
            load_chunk<PREC, TC_BM, KC, 16 / E>(sA, A_BYTES, A, Af, a32, g.ta, g.lda, w.m0, o.M, k0, g.K, alpha);
            load_chunk<PREC, TC_BN, KC, 16 / E>(sB, B_BYTES, B, Bf, b32, g.tb ? 0 : 1, g.ldb, w.n0, o.N, k0, g.K, 1.0f);
            // generic-proxy shared-memory writes -> visible to the tensor core (async proxy)
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncthreads();
            if (tid == 0) {
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t a0 = smem_u32(sA), b0 = smem_u32(sB);
#pragma unroll
                for (int kk = 0; kk < KC / Cfg::KSTEP; ++kk) {
                    const uint32_t koff = kk * Cfg::KSTEP * E / 16 * LBO;
#pragma unroll
                    for (int p = 0; p < Cfg::NPROD; ++p) {
                        // products a_i b_j with i + j <= 2, largest first
                        const int ia = (Cfg::NPROD == 1) ? 0 : (p == 0 ? 0 : p == 1 ? 0 : p == 2 ? 1 : p == 3 ? 0 : p == 4 ? 1 : 2);
                        const int ib = (Cfg::NPROD == 1) ? 0 : (p == 0 ? 0 : p == 1 ? 1 : p == 2 ? 0 : p == 3 ? 2 : p == 4 ? 1 : 0);
                        const uint64_t da = make_sdesc(a0 + ia * A_BYTES + koff, LBO, SBO);
                        const uint64_t db = make_sdesc(b0 + ib * B_BYTES + koff, LBO, SBO);
                        const uint32_t accf = (first && kk == 0 && p == 0) ? 0u : 1u;
                        if constexpr (PREC == QCM_PREC_TF32) {
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}\n"
                                :: "r"(tmem), "l"(da), "l"(db), "r"(IDESC), "r"(accf));
                        } else {
                            asm volatile(
                                "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                                :: "r"(tmem), "l"(da), "l"(db), "r"(IDESC), "r"(accf));
                        }
                    }
                }
                asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                             :: "r"(smem_u32(&mbar[st])) : "memory");
            }
            first = false;
            pending[st] = true;
            ++chunk;
        }
        if (aborted) break;
        // segment complete: wait for its MMAs, then drain TMEM into the FP64 accumulators
        int to = 0;
        for (int i = 0; i < NSTAGE; ++i) {
            if (pending[i]) {
                if (!mbar_wait(smem_u32(&mbar[i]), phase[i])) to = 1;
                phase[i] ^= 1u;
                pending[i] = false;
            }
        }
        if (__syncthreads_or(to)) { aborted = true; break; }
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 16) {
            uint32_t r[16];
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                  "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
                  "=r"(r[15])
                : "r"(trow + (uint32_t)c0));
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float x = __uint_as_float(r[j]);
                const float t = acc_hi[c0 + j] + x;                         // Knuth two-sum
                const float bp = t - acc_hi[c0 + j];
                const float err = (acc_hi[c0 + j] - (t - bp)) + (x - bp);
                acc_hi[c0 + j] = t;
                acc_lo[c0 + j] += err;
            }
        }
        // the next segment's first MMA overwrites TMEM: all reads must be complete
        asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
        __syncthreads();
    }
    if (aborted && tid == 0) atomicExch(&g_tc_status, 1);

    // ---- epilogue: FP64 accumulators -> output tile (written once)
    const bool c32 = (bufs.f32mask >> o.c_buf) & 1u;
    const int64_t row = w.m0 + quad * 32 + lane;
    if (!aborted && row < o.M) {
        if (c32) {
            float* __restrict__ C = (float*)bufs.p[o.c_buf] + o.c_off;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int64_t col = w.n0 + chalf * 32 + j;
                if (col < o.N) C[row + col * o.ldc] = acc_hi[j] + acc_lo[j];
            }
        } else {
            double* __restrict__ C = bufs.p[o.c_buf] + o.c_off;
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                const int64_t col = w.n0 + chalf * 32 + j;
                if (col < o.N) C[row + col * o.ldc] = (double)acc_hi[j] + (double)acc_lo[j];
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"((uint32_t)TC_BN));
    }
}

// Dynamic shared memory per CTA.  Padded to at least 32 KiB so that no more than
// 7 CTAs share an SM: each holds 64 TMEM columns and an SM has 512.
static int tc_smem_bytes(int precision) {
    int slices = (precision == QCM_PREC_BF16X3) ? 3 : 1;
    int need = 2 * slices * (TC_BM + TC_BN) * TC_KB;  // two pipeline stages
    return need < 32768 ? 32768 : need;
}

// Work list for the tensor-core executor: 128 x 64 tiles.
int tc_build_work(const Stage& st, std::vector<int64_t>& w) {
    w.clear();
    for (size_t i = 0; i < st.gout.size(); ++i) {
        const GemmOut& g = st.gout[i];
        for (int64_t m0 = 0; m0 < g.M; m0 += TC_BM)
            for (int64_t n0 = 0; n0 < g.N; n0 += TC_BN) {
                w.push_back((int64_t)i);
                w.push_back(m0);
                w.push_back(n0);
            }
    }
    return QCM_OK;
}

int tc_launch(const void* d_out, const void* d_seg, const void* d_work, int64_t n_work, double* const* bufs,
              uint32_t f32mask, int precision, void* stream) {
    cudaStream_t s = (cudaStream_t)stream;
    if (n_work == 0) return QCM_OK;
    if (n_work > 0x7fffffffLL) { set_error("tensor-core work list too large"); return QCM_E_RANGE; }
    TcBufs tb;
    for (int i = 0; i < QCM_NBUF; ++i) tb.p[i] = bufs[i];
    tb.f32mask = f32mask;
    const int smem = tc_smem_bytes(precision);
    cudaError_t e;
    if (precision == QCM_PREC_TF32) {
        e = cudaFuncSetAttribute(tc_gemm_kernel<QCM_PREC_TF32>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) { set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e)); return QCM_E_CUDA; }
        tc_gemm_kernel<QCM_PREC_TF32><<<(unsigned)n_work, TC_THREADS, smem, s>>>(
            tb, (const TcOut*)d_out, (const TcSeg*)d_seg, (const TcWork*)d_work);
    } else if (precision == QCM_PREC_BF16X3) {
        e = cudaFuncSetAttribute(tc_gemm_kernel<QCM_PREC_BF16X3>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) { set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e)); return QCM_E_CUDA; }
        tc_gemm_kernel<QCM_PREC_BF16X3><<<(unsigned)n_work, TC_THREADS, smem, s>>>(
            tb, (const TcOut*)d_out, (const TcSeg*)d_seg, (const TcWork*)d_work);
    } else {
        set_error("unknown tensor-core precision");
        return QCM_E_INVALID;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(std::string("tc_gemm launch: ") + cudaGetErrorString(e)); return QCM_E_CUDA; }
    return QCM_OK;
}

// ------------------------------------------------------------------ image executor (BF16x3)
// Operands are split once per call into BF16 slice images laid out exactly as
// the MMA reads them from shared memory (ImgPanel).  A persistent kernel, one
// CTA per SM, then runs a warp-specialised pipeline over its share of the
// output tiles: warp 0 (one lane) streams image chunks into TI_NS shared-memory
// stages with cp.async.bulk (completion by transaction count on an mbarrier),
// warp 1 (one lane) issues the six BF16 products per K-step into one of two
// TMEM accumulators, and warps 2..9 drain each finished segment (one block
// product of the split-K sum) into compensated FP32 register sums, scaled by
// the segment's coefficient, and store the tile once.
constexpr int TI_NS = 4;                        // shared-memory stages
constexpr int TI_THREADS = 10 * 32;
constexpr uint32_t TI_SLICE = 16 * 512;         // one slice of a 128-row x 64-byte chunk
constexpr uint32_t TI_STAGE = 6 * TI_SLICE;     // A and B, three slices each
constexpr int TI_EPI_LD = 17;                   // epilogue staging row stride (floats)
// A-resident mode: IMG_ARES_MAX A chunks (three slices each) stay in shared
// memory, followed by TI_NSB stages of B chunks; same footprint as TI_NS stages.
constexpr int TI_NSB = 3;
constexpr uint32_t TI_ACHUNK = 3 * TI_SLICE;
static_assert(IMG_ARES_MAX * TI_ACHUNK + TI_NSB * TI_ACHUNK <= TI_NS * TI_STAGE, "A-resident layout must fit");
constexpr uint32_t TI_SMEM = TI_NS * TI_STAGE + 8 * 32 * TI_EPI_LD * 4 + 1024;
constexpr uint64_t TI_WAIT_NS = 4000000000ull;  // a wait that lasts this long gives up

struct TiArgs {
    int32_t ares;             // A-resident mode (ImgTables::ares)
    const int64_t* cost;      // A-resident mode: prefix sums of the tile costs
    const ImgUnit* units;
    const ImgSeg* segs;
    const ImgOut* outs;
    const uint8_t* img;
    const uint8_t* cimg;      // constant images of the plan (coefficient matrices)
    const int64_t* coltab;    // (offset, ld) pairs of the output tiles of mode-1 outputs
    double* p[QCM_NBUF];
    uint32_t f32mask;
    int32_t n_units;
    int32_t nprod;            // slice products per K-step: 6 (BF16x3) or 3 (BF16x2)
};

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ bool mbar_try(uint32_t mbar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done) : "r"(mbar), "r"(parity) : "memory");
    return done != 0;
}

// Bounded wait: gives up after TI_WAIT_NS, or early when another role of the
// CTA has raised the abort flag (abort == nullptr: no early exit).
__device__ __forceinline__ bool ti_wait(uint32_t mbar, uint32_t parity, const volatile int* abort) {
    uint64_t t0 = 0;
    for (uint32_t it = 0; it < TC_SPIN_LIMIT; ++it) {
        if (mbar_try(mbar, parity)) return true;
        if ((it & 255u) == 255u) {
            if (abort && *abort) return false;
            const uint64_t t = global_ns();
            if (t0 == 0) t0 = t;
            else if (t - t0 > TI_WAIT_NS) return false;
        }
    }
    return false;
}

__device__ __forceinline__ void mbar_arrive(uint32_t mbar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" :: "r"(mbar) : "memory");
}

// Arrive without release semantics.  The epilogue signals with it that its TMEM
// reads of an accumulator are complete (tcgen05.wait::ld / wait::st precede
// it); a release arrive would also wait until all of the warp's earlier global
// stores of output tiles are acknowledged, which serialised the epilogue.
__device__ __forceinline__ void mbar_arrive_relaxed(uint32_t mbar) {
    asm volatile("mbarrier.arrive.relaxed.cta.shared::cta.b64 _, [%0];" :: "r"(mbar) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" :: "r"(mbar), "r"(bytes) : "memory");
}

// global -> shared bulk copy (16-byte aligned addresses, size a multiple of 16)
__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void* src, uint32_t bytes, uint32_t mbar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                 :: "r"(dst), "l"(src), "r"(bytes), "r"(mbar) : "memory");
}

__device__ __forceinline__ void mma_commit(uint32_t mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(mbar)
                 : "memory");
}

// One CTA per (panel, K-chunk): warp w builds 8-row groups w, w+8, ...; lane
// (rr, q) reads the 8 K-values of core matrix q of row rr and writes them as
// one 16-byte vector per slice.
__global__ void __launch_bounds__(256)
build_images_kernel(const ImgPanel* __restrict__ panels, const int32_t* __restrict__ items,
                    const int64_t* __restrict__ gather, uint8_t* __restrict__ img, TcBufs bufs, int nsl) {
    const ImgPanel P = panels[items[2 * blockIdx.x]];
    const int c = items[2 * blockIdx.x + 1];
    const bool f32 = (bufs.f32mask >> P.src_buf) & 1u;
    const int64_t so = P.kcontig == 2 ? 0 : P.src_off;
    const float* __restrict__ S32 = (const float*)bufs.p[P.src_buf] + so;
    const double* __restrict__ S64 = bufs.p[P.src_buf] + so;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int rr = lane & 7, q = lane >> 3;
    const int k0 = c * 32 + q * 8;
    const uint32_t sstride = (uint32_t)P.G * 512u;
    uint8_t* base = img + P.img_off + (size_t)c * 3 * sstride + q * 128 + rr * 16;
    for (int g = warp; g < P.G; g += 8) {
        const int r = g * 8 + rr;
        float v[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int k = k0 + j;
            float x = 0.0f;
            if (r < P.R && k < P.K) {
                if (P.kcontig == 2) {   // column k = one contiguous source tile
                    const int64_t ix = __ldg(gather + P.src_off + k) + r;
                    x = f32 ? __ldg((const float*)bufs.p[P.src_buf] + ix) : (float)__ldg(bufs.p[P.src_buf] + ix);
                } else {
                    const int ix = P.kcontig ? r * P.ld + k : r + k * P.ld;
                    x = f32 ? __ldg(S32 + ix) : (float)__ldg(S64 + ix);
                }
            }
            v[j] = x;
        }
        put_vec<QCM_PREC_BF16X3>(base + (size_t)g * 512, 0, sstride, v, nsl);
    }
}

// This CTA's tiles u = blockIdx.x, blockIdx.x + gridDim.x, ... with the
// descriptors of the next two tiles and of the next tile's first segment
// requested ahead of use, so that no role stalls on a chain of dependent
// global loads at a tile boundary (most K1 tiles have a single short segment).
struct TiCursor {
    const ImgUnit* units;
    const ImgSeg* segs;
    int n, g, u;   // tiles u, u+g, ... below n
    ImgUnit cur, nxt, nn;
    ImgSeg first_cur, first_nxt;

    __device__ static ImgUnit no_unit() {
        ImgUnit e;
        e.out = 0; e.m0 = 0; e.n0 = 0; e.nt = 16; e.s_begin = 0; e.s_end = 0;
        return e;
    }
    __device__ static ImgSeg no_seg() {
        ImgSeg z;
        z.a_img = 0; z.b_img = 0; z.a_G = 1; z.b_G = 1; z.kc = 0; z.alpha = 0.0f; z.flags = 0;
        z.a_panel = 0; z.a_c0 = 0; z.pad = 0;
        return z;
    }
    __device__ ImgUnit at(int x) const { return x < n ? units[x] : no_unit(); }
    __device__ ImgSeg seg(int s, int e) const { return s < e ? segs[s] : no_seg(); }
    // strided (u0 = blockIdx.x, step gridDim.x) or contiguous ([u0, end), step 1) tiles
    __device__ void init(const TiArgs& a, int u0, int end, int step) {
        units = a.units; segs = a.segs; n = end; g = step; u = u0;
        cur = at(u);
        nxt = at(u + g);
        first_cur = seg(cur.s_begin, cur.s_end);
    }
    __device__ bool valid() const { return u < n; }
    __device__ bool has_next() const { return u + g < n; }
    __device__ void prefetch() {
        nn = at(u + 2 * g);
        first_nxt = seg(nxt.s_begin, nxt.s_end);
    }
    __device__ void advance() {
        u += g; cur = nxt; nxt = nn; first_cur = first_nxt;
    }
};

// TMEM columns of one CTA: two accumulators (segments alternate), then the
// compensated running sum (hi, lo) of the tile.
constexpr uint32_t TI_TMEM_COLS = 512;
constexpr uint32_t TI_COL_HI = 256, TI_COL_LO = 384;

__device__ __forceinline__ void tmem_ld16(uint32_t taddr, uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
}

__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t (&r)[16]) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        :: "r"(taddr), "r"(r[0]), "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7]),
           "r"(r[8]), "r"(r[9]), "r"(r[10]), "r"(r[11]), "r"(r[12]), "r"(r[13]), "r"(r[14]), "r"(r[15])
        : "memory");
}

// Store 16 finished columns (c0 .. c0+15 of the tile) of this lane's row.
__device__ __forceinline__ void ti_store16(const TiArgs& a, const ImgOut& O, const ImgUnit& U, int i0, int lane,
                                           int cbase, const float (&hi)[16], const float (&lo)[16], float* stg) {
    const bool c32 = (a.f32mask >> O.c_buf) & 1u;
    float* __restrict__ C32 = (float*)a.p[O.c_buf] + O.c_off;
    double* __restrict__ C64 = a.p[O.c_buf] + O.c_off;
    if (O.mode == 1) {
        // column j is one output tile: element i at (i % rows) + (i / rows)*ld_j of it;
        // with O.pad > 0 the tile is a run of pitch O.rows of which O.pad rows are stored
        const int i = i0 + lane;
        const int64_t ir = i % O.rows, ic = i / O.rows;
        const bool row_ok = O.pad == 0 || ir < O.pad;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int col = U.n0 + cbase + j;
            if (i < O.mrows && col < O.ncols && row_ok) {
                const int64_t off = __ldg(a.coltab + 2 * (O.ctab + col)) + ir + ic * __ldg(a.coltab + 2 * (O.ctab + col) + 1);
                if (c32) ((float*)a.p[O.c_buf])[off] = hi[j] + lo[j];
                else a.p[O.c_buf][off] = (double)hi[j] + (double)lo[j];
            }
        }
    } else if (O.si == 1) {
        // lanes hold consecutive rows i: each column store is coalesced
        const int i = i0 + lane;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int col = U.n0 + cbase + j;
            if (i < O.mrows && col < O.ncols) {
                const int64_t off = (int64_t)i + (int64_t)col * O.sj;
                if (c32) C32[off] = hi[j] + lo[j];
                else C64[off] = (double)hi[j] + (double)lo[j];
            }
        }
    } else if (O.pad == 1 && c32) {
        // as below, for an output whose contiguous direction is padded to a multiple
        // of 4 elements on 16-byte aligned columns (the K1 result): each lane stores
        // 4 consecutive elements, 8 row runs per warp store instead of 2; the
        // elements past ncols land in the padding (they are zero: the operand
        // images are zero-padded)
        const uint32_t sbase = smem_u32(stg);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            asm volatile("st.shared.f32 [%0], %1;" :: "r"(sbase + (uint32_t)((lane * TI_EPI_LD + j) * 4)),
                         "f"(hi[j] + lo[j]) : "memory");
        __syncwarp();
        const int q = lane & 3, r = lane >> 2;
        const int col = U.n0 + cbase + 4 * q;
        float vv[4][4];
#pragma unroll
        for (int k = 0; k < 4; ++k)
#pragma unroll
            for (int e = 0; e < 4; ++e)
                asm volatile("ld.shared.f32 %0, [%1];" : "=f"(vv[k][e])
                             : "r"(sbase + (uint32_t)(((r + 8 * k) * TI_EPI_LD + 4 * q + e) * 4)) : "memory");
        __syncwarp();
        if (col < (O.ncols + 3) / 4 * 4) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const int row = i0 + r + 8 * k;
                if (row < O.mrows)
                    *(float4*)(C32 + (int64_t)row * O.si + col) = make_float4(vv[k][0], vv[k][1], vv[k][2], vv[k][3]);
            }
        }
    } else {
        // rows i lie O.si apart in memory and columns are contiguous: pass the
        // 32 x 16 block through shared memory so that 16 lanes store one row run
        // explicit shared-space accesses (ld/st.shared), so that they need no
        // ordering against the warp's outstanding global stores
        const uint32_t sbase = smem_u32(stg);
#pragma unroll
        for (int j = 0; j < 16; ++j)
            asm volatile("st.shared.f32 [%0], %1;" :: "r"(sbase + (uint32_t)((lane * TI_EPI_LD + j) * 4)),
                         "f"(hi[j] + lo[j]) : "memory");
        __syncwarp();
        const int jj = lane & 15, r0 = lane >> 4;
        const int col = U.n0 + cbase + jj;
        // all 16 shared-memory reads first, then 16 independent stores
        float vv[16];
#pragma unroll
        for (int k = 0; k < 16; ++k)
            asm volatile("ld.shared.f32 %0, [%1];" : "=f"(vv[k])
                         : "r"(sbase + (uint32_t)(((2 * k + r0) * TI_EPI_LD + jj) * 4)) : "memory");
        __syncwarp();
        if (col < O.ncols) {
            const int64_t base = (int64_t)(i0 + r0) * O.si + col;
            const int64_t step = 2 * O.si;
#pragma unroll
            for (int k = 0; k < 16; ++k) {
                if (i0 + r0 + 2 * k < O.mrows) {
                    if (c32) C32[base + k * step] = vv[k];
                    else C64[base + k * step] = (double)vv[k];
                }
            }
        }
    }
}

__global__ void __launch_bounds__(TI_THREADS, 1) tc_img_kernel(TiArgs a) {
    const int nprod = a.nprod;
    const int nsl = nprod == 3 ? 2 : 3;   // image slices the products read (BF16x2: slices 0 and 1)
    extern __shared__ uint8_t ti_smem_raw[];
    uint8_t* smem = (uint8_t*)(((uintptr_t)ti_smem_raw + 1023) & ~(uintptr_t)1023);
    float* epi = (float*)(smem + TI_NS * TI_STAGE);
    __shared__ __align__(8) uint64_t bar_full[TI_NS], bar_empty[TI_NS], bar_accf[2], bar_acce[2], bar_fin;
    __shared__ __align__(8) uint64_t bar_ares_full, bar_ares_empty;
    __shared__ uint32_t tmem_sh;
    __shared__ int abort_sh;
    __shared__ int range_sh[2];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    volatile int* abort_flag = &abort_sh;

    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                     :: "r"(smem_u32(&tmem_sh)), "r"(TI_TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (tid == 32) {
        for (int i = 0; i < TI_NS; ++i) {
            // full: the bulk-copy producer's arrive, completed by its transaction bytes
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar_full[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar_empty[i])));
        }
        for (int i = 0; i < 2; ++i) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar_accf[i])));
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 8;" :: "r"(smem_u32(&bar_acce[i])));
        }
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar_fin)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar_ares_full)));
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" :: "r"(smem_u32(&bar_ares_empty)));
        abort_sh = 0;
        // this CTA's tiles: a contiguous cost-balanced range (A-resident mode), else strided
        if (a.ares) {
            const int64_t total = a.cost[a.n_units];
            int r2[2];
            for (int side = 0; side < 2; ++side) {
                const int64_t target = total * (int64_t)(blockIdx.x + side) / (int64_t)gridDim.x;
                int lo = 0, hi = a.n_units;   // first tile whose cost prefix reaches the target
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (a.cost[mid] < target) lo = mid + 1; else hi = mid;
                }
                r2[side] = lo;
            }
            range_sh[0] = r2[0];
            range_sh[1] = blockIdx.x + 1 == gridDim.x ? a.n_units : r2[1];
        } else {
            range_sh[0] = blockIdx.x;
            range_sh[1] = a.n_units;
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmem_sh;
    const int u_begin = range_sh[0], u_end = range_sh[1];
    const int u_step = a.ares ? 1 : (int)gridDim.x;
    uint8_t* ares_base = smem;                                  // A-resident mode: A chunks ...
    uint8_t* bst_base = smem + IMG_ARES_MAX * TI_ACHUNK;        // ... then the B stages

    if (warp == 0) {
        if (lane == 0) {
            // ---------------- bulk-copy producer
            uint32_t it = 0;
            bool ok = true;
            TiCursor cu;
            cu.init(a, u_begin, u_end, u_step);
            if (a.ares) {
                // A-resident: load a run's A chunks once, then stream the B chunks of its tiles
                int run = -1;
                int64_t key_img = -1;
                int key_m0 = -1;
                for (; cu.valid() && ok; cu.advance()) {
                    cu.prefetch();
                    const ImgUnit U = cu.cur;
                    const ImgSeg S = cu.first_cur;
                    const int gA0 = U.m0 >> 3, gB0 = U.n0 >> 3;
                    if (S.a_img != key_img || U.m0 != key_m0) {
                        if (run >= 0 && !ti_wait(smem_u32(&bar_ares_empty), (uint32_t)run & 1u, abort_flag)) {
                            ok = false;
                            break;
                        }
                        ++run;
                        key_img = S.a_img;
                        key_m0 = U.m0;
                        const uint32_t bA = (uint32_t)min(16, S.a_G - gA0) * 512u;
                        const uint32_t fa = smem_u32(&bar_ares_full);
                        mbar_expect_tx(fa, (uint32_t)nsl * bA * (uint32_t)S.kc);
                        for (int c = 0; c < S.kc; ++c)
                            for (int sl = 0; sl < nsl; ++sl)
                                bulk_g2s(smem_u32(ares_base + c * TI_ACHUNK + sl * TI_SLICE),
                                         a.img + S.a_img + ((int64_t)(c * 3 + sl) * S.a_G + gA0) * 512, bA, fa);
                    }
                    const uint8_t* bbase = (S.flags & IMG_B_CONST) ? a.cimg : a.img;
                    const uint32_t bB = (uint32_t)min(U.nt >> 3, S.b_G - gB0) * 512u;
                    for (int c = 0; c < S.kc; ++c, ++it) {
                        const uint32_t st = it % (uint32_t)TI_NSB, ph = (it / (uint32_t)TI_NSB) & 1u;
                        if (!ti_wait(smem_u32(&bar_empty[st]), ph ^ 1u, abort_flag)) { ok = false; break; }
                        const uint32_t fb = smem_u32(&bar_full[st]);
                        mbar_expect_tx(fb, (uint32_t)nsl * bB);
                        for (int sl = 0; sl < nsl; ++sl)
                            bulk_g2s(smem_u32(bst_base + st * TI_ACHUNK + sl * TI_SLICE),
                                     bbase + S.b_img + ((int64_t)(c * 3 + sl) * S.b_G + gB0) * 512, bB, fb);
                    }
                }
                if (!ok) { *abort_flag = 1; atomicExch(&g_tc_status, 2); }
                // the latest copies of every stage and of the resident A must have landed
                for (uint32_t k = 0; k < (uint32_t)TI_NSB && k < it; ++k) {
                    const uint32_t j = it - 1 - k;
                    if (!ti_wait(smem_u32(&bar_full[j % TI_NSB]), (j / TI_NSB) & 1u, nullptr)) atomicExch(&g_tc_status, 2);
                }
                if (run >= 0 && !ti_wait(smem_u32(&bar_ares_full), (uint32_t)run & 1u, nullptr))
                    atomicExch(&g_tc_status, 2);
            }
            for (; !a.ares && cu.valid() && ok; cu.advance()) {
                cu.prefetch();
                const ImgUnit U = cu.cur;
                const int gA0 = U.m0 >> 3, gB0 = U.n0 >> 3;
                ImgSeg Sn = cu.first_cur;
                for (int s = U.s_begin; s < U.s_end && ok; ++s) {
                    const ImgSeg S = Sn;
                    if (s + 1 < U.s_end) Sn = a.segs[s + 1];
                    const uint8_t* bbase = (S.flags & IMG_B_CONST) ? a.cimg : a.img;
                    const uint32_t bA = (uint32_t)min(16, S.a_G - gA0) * 512u;
                    const uint32_t bB = (uint32_t)min(U.nt >> 3, S.b_G - gB0) * 512u;
                    for (int c = 0; c < S.kc; ++c, ++it) {
                        const uint32_t st = it % (uint32_t)TI_NS, ph = (it / (uint32_t)TI_NS) & 1u;
                        if (!ti_wait(smem_u32(&bar_empty[st]), ph ^ 1u, abort_flag)) { ok = false; break; }
                        const uint32_t fb = smem_u32(&bar_full[st]);
                        mbar_expect_tx(fb, (uint32_t)nsl * (bA + bB));
                        const uint32_t dst = smem_u32(smem + st * TI_STAGE);
                        for (int sl = 0; sl < nsl; ++sl) {
                            bulk_g2s(dst + sl * TI_SLICE,
                                     a.img + S.a_img + ((int64_t)(c * 3 + sl) * S.a_G + gA0) * 512, bA, fb);
                            bulk_g2s(dst + (3 + sl) * TI_SLICE,
                                     bbase + S.b_img + ((int64_t)(c * 3 + sl) * S.b_G + gB0) * 512, bB, fb);
                        }
                    }
                }
            }
            if (!a.ares) {
                if (!ok) { *abort_flag = 1; atomicExch(&g_tc_status, 2); }
                // the copies of every stage's latest round must have landed before the CTA exits
                for (uint32_t k = 0; k < (uint32_t)TI_NS && k < it; ++k) {
                    const uint32_t j = it - 1 - k;
                    if (!ti_wait(smem_u32(&bar_full[j % TI_NS]), (j / TI_NS) & 1u, nullptr)) atomicExch(&g_tc_status, 2);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---------------- MMA issuer
            uint32_t it = 0, sc = 0;
            bool ok = true;
            TiCursor cu;
            cu.init(a, u_begin, u_end, u_step);
            if (a.ares) {
                int run = -1;
                int64_t key_img = -1;
                int key_m0 = -1;
                for (; cu.valid() && ok; cu.advance()) {
                    cu.prefetch();
                    const ImgUnit U = cu.cur;
                    const ImgSeg S = cu.first_cur;
                    const uint32_t idesc = make_idesc(1u, TC_BM, U.nt);
                    if (S.a_img != key_img || U.m0 != key_m0) {
                        ++run;
                        key_img = S.a_img;
                        key_m0 = U.m0;
                        if (!ti_wait(smem_u32(&bar_ares_full), (uint32_t)run & 1u, abort_flag)) { ok = false; break; }
                    }
                    const uint32_t b = sc & 1u;
                    if (!ti_wait(smem_u32(&bar_acce[b]), ((sc >> 1) & 1u) ^ 1u, abort_flag)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t d = tmem + b * 128u;
                    for (int c = 0; c < S.kc; ++c, ++it) {
                        const uint32_t st = it % (uint32_t)TI_NSB, ph = (it / (uint32_t)TI_NSB) & 1u;
                        if (!ti_wait(smem_u32(&bar_full[st]), ph, abort_flag)) { ok = false; break; }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t a0 = smem_u32(ares_base + c * TI_ACHUNK), b0 = smem_u32(bst_base + st * TI_ACHUNK);
                        const uint64_t da0 = make_sdesc(a0, 128, 512), db0 = make_sdesc(b0, 128, 512);
#pragma unroll
                        for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
                            for (int p = 0; p < 6; ++p) {
                                if (p >= nprod) break;   // BF16x2 form: the slice pairs with i + j <= 1
                                const int ia = p == 2 ? 1 : p == 4 ? 1 : p == 5 ? 2 : 0;
                                const int ib = p == 1 ? 1 : p == 3 ? 2 : p == 4 ? 1 : 0;
                                // start-address field (bits 0-13, address >> 4) advanced by the offset
                                const uint64_t da = da0 + (uint64_t)((ia * TI_SLICE + kk * 256) >> 4);
                                const uint64_t db = db0 + (uint64_t)((ib * TI_SLICE + kk * 256) >> 4);
                                const uint32_t accum = (c == 0 && kk == 0 && p == 0) ? 0u : 1u;
                                asm volatile(
                                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                                    :: "r"(d), "l"(da), "l"(db), "r"(idesc), "r"(accum));
                            }
                        }
                        mma_commit(smem_u32(&bar_empty[st]));
                    }
                    if (!ok) break;
                    mma_commit(smem_u32(&bar_accf[b]));
                    ++sc;
                    // the run ends here when the next tile reads another A tile: release the resident A
                    if (!cu.has_next() || cu.first_nxt.a_img != key_img || cu.nxt.m0 != key_m0)
                        mma_commit(smem_u32(&bar_ares_empty));
                }
            }
            for (; !a.ares && cu.valid() && ok; cu.advance()) {
                cu.prefetch();
                const ImgUnit U = cu.cur;
                const uint32_t idesc = make_idesc(1u, TC_BM, U.nt);
                int kcn = cu.first_cur.kc;
                for (int s = U.s_begin; s < U.s_end && ok; ++s) {
                    const int kc = kcn;
                    if (s + 1 < U.s_end) kcn = a.segs[s + 1].kc;
                    const uint32_t b = sc & 1u;
                    if (!ti_wait(smem_u32(&bar_acce[b]), ((sc >> 1) & 1u) ^ 1u, abort_flag)) { ok = false; break; }
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint32_t d = tmem + b * 128u;
                    for (int c = 0; c < kc; ++c, ++it) {
                        const uint32_t st = it % (uint32_t)TI_NS, ph = (it / (uint32_t)TI_NS) & 1u;
                        if (!ti_wait(smem_u32(&bar_full[st]), ph, abort_flag)) { ok = false; break; }
                        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                        const uint32_t a0 = smem_u32(smem + st * TI_STAGE), b0 = a0 + 3 * TI_SLICE;
                        const uint64_t da0 = make_sdesc(a0, 128, 512), db0 = make_sdesc(b0, 128, 512);
#pragma unroll
                        for (int kk = 0; kk < 2; ++kk) {
#pragma unroll
                            for (int p = 0; p < 6; ++p) {
                                if (p >= nprod) break;   // BF16x2 form: the slice pairs with i + j <= 1
                                const int ia = p == 2 ? 1 : p == 4 ? 1 : p == 5 ? 2 : 0;
                                const int ib = p == 1 ? 1 : p == 3 ? 2 : p == 4 ? 1 : 0;
                                // start-address field (bits 0-13, address >> 4) advanced by the offset
                                const uint64_t da = da0 + (uint64_t)((ia * TI_SLICE + kk * 256) >> 4);
                                const uint64_t db = db0 + (uint64_t)((ib * TI_SLICE + kk * 256) >> 4);
                                const uint32_t accum = (c == 0 && kk == 0 && p == 0) ? 0u : 1u;
                                asm volatile(
                                    "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
                                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
                                    :: "r"(d), "l"(da), "l"(db), "r"(idesc), "r"(accum));
                            }
                        }
                        mma_commit(smem_u32(&bar_empty[st]));
                    }
                    if (!ok) break;
                    mma_commit(smem_u32(&bar_accf[b]));
                    ++sc;
                }
            }
            if (!ok) { *abort_flag = 1; atomicExch(&g_tc_status, 2); }
            // every MMA issued must be complete before TMEM is released
            mma_commit(smem_u32(&bar_fin));
            if (!ti_wait(smem_u32(&bar_fin), 0u, nullptr)) atomicExch(&g_tc_status, 2);
        }
    } else {
        // ---------------- epilogue: warps 2..9; TMEM lanes 32*(warp%4).., columns 64*h..
        // Each finished segment is scaled by its coefficient and added into the
        // tile's compensated FP32 sum (Knuth two-sum; hi and lo kept in TMEM).
        const int e = warp - 2, q = warp & 3, h = e >> 2;
        float* stg = epi + e * 32 * TI_EPI_LD;
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)(h * 64);
        uint32_t sc = 0;
        bool ok = true;
        TiCursor cu;
        cu.init(a, u_begin, u_end, u_step);
        ImgOut On = a.outs[cu.cur.out];
        for (; cu.valid() && ok; cu.advance()) {
            cu.prefetch();
            const ImgUnit U = cu.cur;
            const ImgOut O = On;
            On = a.outs[cu.nxt.out];   // the next tile's output descriptor, ahead of use
            const int ncw = max(0, min(64, U.nt - h * 64));
            const int i0 = U.m0 + q * 32;
            float alpha_n = cu.first_cur.alpha;
            if (U.s_begin == U.s_end) {
                // no segment: the tile is zero
                float z[16];
#pragma unroll
                for (int j = 0; j < 16; ++j) z[j] = 0.0f;
                for (int c16 = 0; c16 < 4; ++c16)
                    if (c16 * 16 < ncw) ti_store16(a, O, U, i0, lane, h * 64 + c16 * 16, z, z, stg);
                continue;
            }
            if (U.s_end - U.s_begin == 1) {
                // one segment: no running sum; TMEM loads are issued two at a time
                const float alpha = alpha_n;
                const uint32_t b = sc & 1u;
                ok = __all_sync(0xffffffffu, ti_wait(smem_u32(&bar_accf[b]), (sc >> 1) & 1u, abort_flag));
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
                for (int c32 = 0; c32 < 4; c32 += 2) {
                    if (c32 * 16 >= ncw) break;
                    uint32_t r2[2][16];
#pragma unroll
                    for (int q2 = 0; q2 < 2; ++q2)
                        if ((c32 + q2) * 16 < ncw) tmem_ld16(lane_base + b * 128u + (uint32_t)((c32 + q2) * 16), r2[q2]);
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                    for (int q2 = 0; q2 < 2; ++q2) {
                        if ((c32 + q2) * 16 < ncw) {
                            float hi[16], lo[16];
#pragma unroll
                            for (int j = 0; j < 16; ++j) { hi[j] = alpha * __uint_as_float(r2[q2][j]); lo[j] = 0.0f; }
                            ti_store16(a, O, U, i0, lane, h * 64 + (c32 + q2) * 16, hi, lo, stg);
                        }
                    }
                }
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive_relaxed(smem_u32(&bar_acce[b]));
                ++sc;
                continue;
            }
            for (int s = U.s_begin; s < U.s_end; ++s) {
                const float alpha = alpha_n;
                if (s + 1 < U.s_end) alpha_n = a.segs[s + 1].alpha;
                const bool first = s == U.s_begin, last = s + 1 == U.s_end;
                const uint32_t b = sc & 1u;
                ok = __all_sync(0xffffffffu, ti_wait(smem_u32(&bar_accf[b]), (sc >> 1) & 1u, abort_flag));
                if (!ok) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll 1
                for (int c16 = 0; c16 < 4; ++c16) {
                    if (c16 * 16 >= ncw) break;
                    const uint32_t col = (uint32_t)(c16 * 16);
                    uint32_t r[16];
                    tmem_ld16(lane_base + b * 128u + col, r);
                    float hi[16], lo[16];
                    if (first) {
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int j = 0; j < 16; ++j) { hi[j] = alpha * __uint_as_float(r[j]); lo[j] = 0.0f; }
                    } else {
                        uint32_t rh[16], rl[16];
                        tmem_ld16(lane_base + TI_COL_HI + col, rh);
                        tmem_ld16(lane_base + TI_COL_LO + col, rl);
                        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
                        for (int j = 0; j < 16; ++j) {
                            const float x = alpha * __uint_as_float(r[j]);
                            const float hh = __uint_as_float(rh[j]);
                            const float t = hh + x;  // Knuth two-sum
                            const float bp = t - hh;
                            const float err = (hh - (t - bp)) + (x - bp);
                            hi[j] = t;
                            lo[j] = __uint_as_float(rl[j]) + err;
                        }
                    }
                    if (last) {
                        ti_store16(a, O, U, i0, lane, h * 64 + c16 * 16, hi, lo, stg);
                    } else {
                        uint32_t wh[16], wl[16];
#pragma unroll
                        for (int j = 0; j < 16; ++j) { wh[j] = __float_as_uint(hi[j]); wl[j] = __float_as_uint(lo[j]); }
                        tmem_st16(lane_base + TI_COL_HI + col, wh);
                        tmem_st16(lane_base + TI_COL_LO + col, wl);
                    }
                }
                asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
                asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive_relaxed(smem_u32(&bar_acce[b]));
                ++sc;
            }
        }
        if (!ok && lane == 0) { *abort_flag = 1; atomicExch(&g_tc_status, 2); }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0) {
        __syncwarp();
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(tmem), "r"(TI_TMEM_COLS));
    }
}

static int sm_count_of_current_device() {
    static int cached[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (cached[dev] == 0) {
        int n = 0;
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 152;
        cached[dev] = n;
    }
    return cached[dev];
}

int tc_img_launch(const Stage& st, double* const* bufs, uint32_t f32mask, void* stream, int nprod) {
    if (nprod != 3 && nprod != 6) { set_error("image executor: 3 or 6 slice products"); return QCM_E_INVALID; }
    cudaStream_t s = (cudaStream_t)stream;
    const ImgTables& t = st.img;
    if (t.units.empty()) return QCM_OK;
    if (!st.d_iunit || !bufs[QCM_BUF_IMG]) { set_error("image executor: tables or image buffer missing"); return QCM_E_STATE; }
    TcBufs tb;
    for (int i = 0; i < QCM_NBUF; ++i) tb.p[i] = bufs[i];
    tb.f32mask = f32mask;
    uint8_t* img = (uint8_t*)bufs[QCM_BUF_IMG];
    const size_t n_build = t.build.size() / 2;
    if (n_build > 0)
        build_images_kernel<<<(unsigned)n_build, 256, 0, s>>>((const ImgPanel*)st.d_ipanel, (const int32_t*)st.d_ibuild,
                                                              (const int64_t*)st.d_igather, img, tb,
                                                              nprod == 3 ? 2 : 3);
    cudaError_t e = cudaFuncSetAttribute(tc_img_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TI_SMEM);
    if (e != cudaSuccess) { set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e)); return QCM_E_CUDA; }
    TiArgs a;
    a.units = (const ImgUnit*)st.d_iunit;
    a.segs = (const ImgSeg*)st.d_iseg;
    a.outs = (const ImgOut*)st.d_iout;
    a.img = img;
    a.cimg = (const uint8_t*)st.d_icimg;
    a.ares = t.ares ? 1 : 0;
    a.cost = (const int64_t*)st.d_icost;
    a.coltab = (const int64_t*)st.d_icoltab;
    for (int i = 0; i < QCM_NBUF; ++i) a.p[i] = bufs[i];
    a.f32mask = f32mask;
    a.n_units = (int32_t)t.units.size();
    a.nprod = nprod;
    const int grid = (int)std::min<size_t>(t.units.size(), (size_t)sm_count_of_current_device());
    tc_img_kernel<<<grid, TI_THREADS, TI_SMEM, s>>>(a);
    e = cudaGetLastError();
    if (e != cudaSuccess) { set_error(std::string("tc_img launch: ") + cudaGetErrorString(e)); return QCM_E_CUDA; }
    return QCM_OK;
}

}  // namespace qcm

extern "C" int qcm_device_status(int32_t* status) {
    if (!status) { qcm::set_error("null status"); return QCM_E_INVALID; }
    int v = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&v, qcm::g_tc_status, sizeof(int));
    if (e != cudaSuccess) { qcm::set_error(std::string("cudaMemcpyFromSymbol: ") + cudaGetErrorString(e)); return QCM_E_CUDA; }
    *status = v;
    return QCM_OK;
}
