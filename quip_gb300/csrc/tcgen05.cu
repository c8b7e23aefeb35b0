// tcgen05.cu -- K5 mixed path: the sparse-GP kernel GEMMs on Blackwell tensor cores.
//
//   GEMM1  K = Q X^T   [nc x M]  fused epilogue: W = coef zeta K^(zeta-1) and per-tile
//                                 row sums of coef K^zeta (the local energies)
//   GEMM2  G = W X     [nc x D]  (dE/dq of every centre)
// Operand encodings, all with FP32 accumulation in TMEM:
//   bf16x3: every operand is split x = hi + lo (bf16 each) and the product is
//           hi*hi + hi*lo + lo*hi (three tcgen05.mma kind::f16 per k-step; the dropped
//           lo*lo term is 2^-16 relative);
//   tf32:   operands rounded to TF32 (cvt.rna), one tcgen05.mma kind::tf32 per k-step;
//   f16:    FP16 operands (the TF32 mode's default where the model allows): GEMM1 on FP16
//           descriptors and sparse points, writing W' = S K^(zeta-1) in FP16; GEMM2 on W'
//           and X' = (coef zeta / S) x -- 10-bit mantissas like TF32, in FP16's normal
//           range by construction, at twice the TF32 tensor rate.
// Two kernels: k_tc_gemm (one CTA per 128-row tile) and k_tc_gemm_pair (a cluster of two
// CTAs per 256-row tile, tcgen05 cta_group::2; the only one for FP16), chosen per shape by
// the autotuner.  Both are persistent and warp-specialised (192 threads, one CTA per SM,
// looping over the output tiles):
//   warp 0 lane 0  TMA producer: 2-D tiled loads, 128B swizzle, into an S-stage ring
//   warp 1         TMEM owner (512 columns: two accumulator buffers); lane 0 issues
//                  tcgen05.mma from shared-memory descriptors, tcgen05.commit frees each
//                  stage and hands a finished accumulator buffer to the epilogue
//   warps 2-5      epilogue: tcgen05.ld 32x32b (warp w reads TMEM lanes 32(w%4)..+31),
//                  overlapped with the MMAs of the next tile in the other buffer
// Every mbarrier wait is bounded; on expiry the kernel records an error code, waits
// (bounded) for its own TMA loads and MMAs in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>
#include <map>
#include <mutex>
#include <tuple>

#include "context.h"

namespace gapgpu {
namespace {

constexpr int BM = 128, THREADS = 192;
constexpr int MODE_BF16X3 = 1, MODE_TF32 = 2, MODE_F16 = 3;  // F16: both operands FP16 (CTA pairs only)
constexpr int EPI_KERNEL = 1, EPI_STORE = 2;
// Every mbarrier wait gives up after WAIT_NS of GPU time (%globaltimer), far above any
// legitimate wait of these kernels (a pipeline stage or an accumulator buffer: microseconds).
constexpr unsigned long long WAIT_NS = 250ull * 1000 * 1000;
constexpr int SMEM_BUDGET = 200 * 1024;
constexpr int TMEM_COLS = 512;   // two accumulator buffers, ACC_STRIDE columns apart
constexpr int ACC_STRIDE = 256;

// Stage layout for one k-chunk of 128 bytes per operand row: NOPS planes (hi, lo) of A
// (BM rows) then NOPS planes of B (BN rows).
template <int MODE, int BN>
struct Cfg {
    static constexpr int KB = MODE == MODE_BF16X3 ? 64 : 32;  // k elements per stage
    static constexpr int NOPS = MODE == MODE_BF16X3 ? 2 : 1;
    static constexpr int TILE_A = BM * 128;
    static constexpr int TILE_B = BN * 128;
    static constexpr int STAGE = NOPS * (TILE_A + TILE_B);
    static constexpr int STAGES = SMEM_BUDGET / STAGE > 8 ? 8 : SMEM_BUDGET / STAGE;
    static constexpr int KSTEP = MODE == MODE_BF16X3 ? 16 : 8;  // k per tcgen05.mma
    static_assert(STAGES >= 2, "stage ring too small");
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}
__device__ __forceinline__ bool mbar_try(uint64_t* b, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(su32(b)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait.  Gives up after WAIT_NS nanoseconds of GPU time, or as soon as another
// thread of the CTA has given up (abort flag in shared memory).  The clock is read every
// 64 polls (try_wait itself may suspend the thread for a short while).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, int* err, int code,
                                          unsigned long long limit_ns = WAIT_NS) {
    if (mbar_try(b, parity)) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned i = 1;; ++i) {
        if (mbar_try(b, parity)) return true;
        if ((i & 63) == 0) {
            if (*abort_flag) return false;
            if (global_ns() - t0 > limit_ns) break;
        }
    }
    *abort_flag = 1;
    atomicOr(err, code);
    return false;
}

// Diagnostic: one warp waits on an mbarrier that nothing arrives on, with the bounded
// wait of the GEMM kernels and a caller-chosen time limit; on expiry it records the error
// code and returns.  No asynchronous copy or MMA is in flight.
__global__ void k_wait_probe(unsigned long long limit_ns, int* err) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ volatile int abort_flag;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    mbar_wait(&bar, 0, &abort_flag, err, 8, limit_ns);  // on expiry: err |= 8
}

// 2-D tiled TMA load with an L2 cache policy (createpolicy): the operand every CTA
// re-reads (the sparse points) is kept in L2, the streamed one is evicted first.
__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* tm, int c0, int c1, uint64_t* bar, uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1, {%2, %3}], "
        "[%4], %5;" ::"r"(su32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(su32(bar)), "l"(policy)
        : "memory");
}
__device__ __forceinline__ uint64_t policy_evict_last() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}

__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    // K-major operand, 128-byte swizzle, 8-row groups 1024 bytes apart (SBO), version 1.
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFF);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

template <int MODE, int BN>
__device__ __forceinline__ constexpr uint32_t idesc() {
    // D = F32 (bit 4); A/B format bits 7-9 / 10-12 (BF16 = 1 for kind::f16, TF32 = 2 for
    // kind::tf32); K-major A and B; N >> 3 at bits 17-22; M >> 4 at bits 24-28.
    return (1u << 4) | ((MODE == MODE_BF16X3 ? 1u : 2u) << 7) | ((MODE == MODE_BF16X3 ? 1u : 2u) << 10) |
           ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <int MODE, int BN>
__device__ __forceinline__ void mma(uint32_t dt, uint64_t a, uint64_t b, uint32_t acc) {
    if constexpr (MODE == MODE_BF16X3)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
            "l"(a), "l"(b), "r"(idesc<MODE, BN>()), "r"(acc));
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
            "l"(a), "l"(b), "r"(idesc<MODE, BN>()), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar)) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

struct EpiParams {
    int rows;             // valid rows (centres)
    int ldo;              // leading dimension of the outputs
    const float* coef;    // [N] alpha * sparseCutoff * delta^2   (EPI_KERNEL)
    float zeta;
    int izeta;
    void* out_hi;         // W (bf16 hi or tf32 fp32) / G (fp32)
    void* out_lo;         // W lo (bf16x3)
    double* epart;        // [ntiles x rows]: energies per 64-column block (rows fastest)
    int ntiles;
    int w_f16;            // EPI_KERNEL, TF32: write W' = wscale K^(zeta-1) as FP16 (for the FP16 second GEMM)
    float wscale;
};

// Kernel function of one row's 32-column block: e += coef K^zeta and w = coef zeta K^(zeta-1)
// (TF32-rounded when tf32_round) or W' = wscale K^(zeta-1) for the FP16 second GEMM.  The
// zeta = 4 test is taken once per block, not per element: the unrolled common path is then
// one contiguous stretch of code (with the other exponents interleaved per element, the
// epilogue warps were held up by instruction fetch).
__device__ __forceinline__ void kernel_block(const EpiParams& ep, int col0, const float* v, float& e_acc, float* w,
                                             bool tf32_round) {
    if (ep.izeta == 4) {
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float k = v[j], cf = ep.coef[col0 + j], km1 = k * k * k;
            e_acc += cf * km1 * k;
            const float x = cf * ep.zeta * km1;
            w[j] = ep.w_f16 ? ep.wscale * km1 : (tf32_round ? round_tf32(x) : x);
        }
    } else {  // unrolled too: w and v stay in registers (this block is not executed for zeta = 4)
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float k = v[j], cf = ep.coef[col0 + j];
            float km1;
            if (ep.izeta > 0) { km1 = 1.f; for (int t = 1; t < ep.izeta; ++t) km1 *= k; }
            else km1 = powf(k, ep.zeta - 1.f);
            e_acc += cf * km1 * k;
            const float x = cf * ep.zeta * km1;
            w[j] = ep.w_f16 ? ep.wscale * km1 : (tf32_round ? round_tf32(x) : x);
        }
    }
}

// Epilogue of one 32-column chunk for one row: kernel function and W store (EPI_KERNEL)
// or plain FP32 store (EPI_STORE).
template <int MODE, int EPI>
__device__ __forceinline__ void epilogue_chunk(const EpiParams& ep, int row, int col0, const float* v, float& e_acc) {
    if constexpr (EPI == EPI_KERNEL) {
        float w[32];
        kernel_block(ep, col0, v, e_acc, w, false);
        if constexpr (MODE == MODE_BF16X3) {
            __nv_bfloat16 hi[32], lo[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                hi[j] = __float2bfloat16_rn(w[j]);
                lo[j] = __float2bfloat16_rn(w[j] - __bfloat162float(hi[j]));
            }
            uint4* oh = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(ep.out_hi) + (size_t)row * ep.ldo + col0);
            uint4* ol = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(ep.out_lo) + (size_t)row * ep.ldo + col0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                __stcs(oh + q, reinterpret_cast<const uint4*>(hi)[q]);
                __stcs(ol + q, reinterpret_cast<const uint4*>(lo)[q]);
            }
        } else if (ep.w_f16) {
            // W' = wscale K^(zeta-1) (coef zeta / wscale is folded into the FP16 sparse points)
            __half h[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) h[j] = __float2half_rn(w[j]);
            uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<__half*>(ep.out_hi) + (size_t)row * ep.ldo + col0);
#pragma unroll
            for (int q = 0; q < 4; ++q) __stcs(o + q, reinterpret_cast<const uint4*>(h)[q]);
        } else {
            float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(ep.out_hi) + (size_t)row * ep.ldo + col0);
#pragma unroll
            for (int q = 0; q < 8; ++q)
                __stcs(o + q, make_float4(round_tf32(w[4 * q]), round_tf32(w[4 * q + 1]), round_tf32(w[4 * q + 2]),
                                          round_tf32(w[4 * q + 3])));
        }
    } else {
        float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(ep.out_hi) + (size_t)row * ep.ldo + col0);
#pragma unroll
        for (int q = 0; q < 8; ++q) __stcs(o + q, make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]));
    }
}

// TF32 epilogue of one 32 x 32 block of a warp (row row0 + lane in this thread) through
// its 4 KB shared-memory stage: each thread writes its row (16-byte chunks XOR-swizzled
// by the row, conflict-free), then every store instruction writes 4 rows x 128
// contiguous bytes instead of 32 scattered 16-byte pieces.
template <int EPI>
__device__ __forceinline__ void epilogue_chunk_staged(const EpiParams& ep, int row0, int lane, int col0, const float* v,
                                                      float& e_acc, float* stg) {
    float w[32];
    if constexpr (EPI == EPI_KERNEL) {
        kernel_block(ep, col0, v, e_acc, w, true);
        if (ep.w_f16) {
            // W' rows of 32 FP16 values (64 bytes): 16-byte chunk c of row r at c ^ ((r >> 1) & 3)
            // (conflict-free), then every store instruction writes 8 rows x 64 contiguous bytes
            __half h[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) h[j] = __float2half_rn(w[j]);
            uint4* hrow = reinterpret_cast<uint4*>(reinterpret_cast<char*>(stg) + lane * 64);
#pragma unroll
            for (int c = 0; c < 4; ++c) hrow[c ^ ((lane >> 1) & 3)] = reinterpret_cast<const uint4*>(h)[c];
            __syncwarp();
            __half* hout = reinterpret_cast<__half*>(ep.out_hi);
            const int c = lane & 3;
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int r = 8 * i + (lane >> 2);
                const uint4 val = reinterpret_cast<const uint4*>(reinterpret_cast<const char*>(stg) + r * 64)[c ^ ((r >> 1) & 3)];
                if (row0 + r < ep.rows) __stcs(reinterpret_cast<uint4*>(hout + (size_t)(row0 + r) * ep.ldo + col0) + c, val);
            }
            __syncwarp();
            return;
        }
    } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) w[j] = v[j];
    }
    float4* srow = reinterpret_cast<float4*>(stg + lane * 32);
#pragma unroll
    for (int c = 0; c < 8; ++c) srow[c ^ (lane & 7)] = make_float4(w[4 * c], w[4 * c + 1], w[4 * c + 2], w[4 * c + 3]);
    __syncwarp();
    float* out = reinterpret_cast<float*>(ep.out_hi);
    const int c = lane & 7;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const int r = 4 * i + (lane >> 3);
        const float4 val = reinterpret_cast<const float4*>(stg + r * 32)[c ^ (r & 7)];
        if (row0 + r < ep.rows) __stcs(reinterpret_cast<float4*>(out + (size_t)(row0 + r) * ep.ldo + col0) + c, val);
    }
    __syncwarp();  // the stage is rewritten by the next block
}

// C[m, n] = sum_k A[m, k] B[n, k] over m_tiles x n_tiles output tiles of BM x BN.
template <int MODE, int EPI, int BN>
__global__ void __launch_bounds__(THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tA0, const __grid_constant__ CUtensorMap tA1,
              const __grid_constant__ CUtensorMap tB0, const __grid_constant__ CUtensorMap tB1, int m_tiles, int n_tiles,
              int kchunks, EpiParams ep, int* err) {
    using C = Cfg<MODE, BN>;
    constexpr int S = C::STAGES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[S], empty[S], tfull[2], tempty[2], drain;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = m_tiles * n_tiles;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], 4); }
        mbar_init(&drain, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        const uint64_t pol_a = policy_evict_first(), pol_b = policy_evict_last();
        int it = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x) {
            const int m0 = (tile / n_tiles) * BM, n0 = (tile % n_tiles) * BN;
            for (int kc = 0; kc < kchunks; ++kc, ++it) {
                const int s = it % S;
                if (it >= S && !mbar_wait(&empty[s], ((it / S) - 1) & 1, &abort_flag, err, 1)) { ok = false; break; }
                unsigned char* st = smem + (size_t)s * C::STAGE;
                mbar_expect_tx(&full[s], C::STAGE);
                const int kx = kc * C::KB;
                tma_load(st, &tA0, kx, m0, &full[s], pol_a);
                if constexpr (MODE == MODE_BF16X3) tma_load(st + C::TILE_A, &tA1, kx, m0, &full[s], pol_a);
                unsigned char* sb = st + C::NOPS * C::TILE_A;
                tma_load(sb, &tB0, kx, n0, &full[s], pol_b);
                if constexpr (MODE == MODE_BF16X3) tma_load(sb + C::TILE_B, &tB1, kx, n0, &full[s], pol_b);
            }
        }
        if (!ok) {  // let the loads already issued land before the CTA exits
            for (int j = it - 1; j >= 0 && j >= it - S; --j)
                mbar_wait(&full[j % S], (j / S) & 1, &abort_flag, err, 0);
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        int it = 0, t = 0;
        bool ok = true;
        for (int tile = blockIdx.x; tile < ntiles && ok; tile += gridDim.x, ++t) {
            const int buf = t & 1;
            if (t >= 2 && !mbar_wait(&tempty[buf], ((t >> 1) - 1) & 1, &abort_flag, err, 2)) break;
            fence_after();
            const uint32_t acc_addr = tmem + buf * ACC_STRIDE;
            for (int kc = 0; kc < kchunks; ++kc, ++it) {
                const int s = it % S;
                if (!mbar_wait(&full[s], (it / S) & 1, &abort_flag, err, 2)) { ok = false; break; }
                fence_after();
                const uint32_t base = su32(smem + (size_t)s * C::STAGE);
                const uint32_t bbase = base + C::NOPS * C::TILE_A;
#pragma unroll
                for (int kk = 0; kk < C::KB / C::KSTEP; ++kk) {
                    const uint32_t koff = kk * 32;  // 32 bytes of K per instruction
                    const uint32_t acc = (kc > 0 || kk > 0) ? 1u : 0u;
                    if constexpr (MODE == MODE_BF16X3) {
                        const uint64_t ah = sdesc(base + koff), al = sdesc(base + C::TILE_A + koff);
                        const uint64_t bh = sdesc(bbase + koff), bl = sdesc(bbase + C::TILE_B + koff);
                        mma<MODE, BN>(acc_addr, ah, bh, acc);
                        mma<MODE, BN>(acc_addr, ah, bl, 1u);
                        mma<MODE, BN>(acc_addr, al, bh, 1u);
                    } else {
                        mma<MODE, BN>(acc_addr, sdesc(base + koff), sdesc(bbase + koff), acc);
                    }
                }
                mma_commit(&empty[s]);
            }
            if (ok) mma_commit(&tfull[buf]);
        }
        mma_commit(&drain);  // arrives once every MMA issued above has completed
        mbar_wait(&drain, 0, &abort_flag, err, 0);
    } else if (warp >= 2) {
        // ---------------- epilogue (warps 2-5; TMEM lane quarter = warp % 4)
        const int q = warp & 3;
        int t = 0;
        for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++t) {
            const int buf = t & 1;
            const int m0 = (tile / n_tiles) * BM, n0 = (tile % n_tiles) * BN;
            if (!mbar_wait(&tfull[buf], (t >> 1) & 1, &abort_flag, err, 4)) break;
            fence_after();
            const int row = m0 + q * 32 + lane;
            float e_acc = 0.f;
#pragma unroll 1
            for (int cc = 0; cc < BN / 32; ++cc) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_STRIDE + cc * 32, v);
                if (row < ep.rows) epilogue_chunk<MODE, EPI>(ep, row, n0 + cc * 32, v, e_acc);
                if constexpr (EPI == EPI_KERNEL) {
                    // energies per 64-column block, whatever the tile width: the sum does not
                    // depend on the autotuner's choice
                    if (cc & 1) {
                        if (row < ep.rows) ep.epart[(size_t)((n0 + cc * 32) / 64) * ep.rows + row] = (double)e_acc;
                        e_acc = 0.f;
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[buf]);
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

// ---------------------------------------------------------------- CTA pairs (TF32)
// The same GEMM on 256-row tiles computed by a cluster of two CTAs (tcgen05
// cta_group::2): each CTA loads its 128 rows of A and half of the BN rows of B, the
// leader (cluster rank 0) issues one 256 x BN x 8 MMA per k-step that reads both CTAs'
// shared memory and writes each CTA's accumulator rows into that CTA's TMEM.  Per SM the
// shared-memory operand traffic per MAC drops from (128 + BN) to (128 + BN / 2) rows.
//   full[s]   leader only: both CTAs' TMA loads complete on it (expect-tx of both)
//   empty[s]  both: the leader's commit arrives on the pair (multicast)
//   tfull[b]  both: accumulator buffer b ready (multicast commit)
//   tempty[b] leader only: 4 epilogue warps of each CTA arrive (remote for the peer)
__device__ __forceinline__ uint32_t cluster_rank() {
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ void cluster_sync_all() {
    asm volatile("barrier.cluster.arrive.release;\n barrier.cluster.wait.acquire;" ::: "memory");
}
// shared::cluster address of the same shared-memory location in CTA `rank` of the cluster
__device__ __forceinline__ uint32_t mapa_rank(uint32_t saddr, uint32_t rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(saddr), "r"(rank));
    return r;
}
__device__ __forceinline__ void mbar_arrive_cluster(uint32_t caddr) {
    asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];" ::"r"(caddr) : "memory");
}
__device__ __forceinline__ void tma_load_pair(void* dst, const CUtensorMap* tm, int c0, int c1, uint32_t bar_cluster,
                                              uint64_t policy) {
    asm volatile(
        "cp.async.bulk.tensor.2d.cta_group::2.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], "
        "[%1, {%2, %3}], [%4], %5;" ::"r"(su32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(bar_cluster), "l"(policy)
        : "memory");
}
// F32 accumulator, A/B format TF32 (2, kind::tf32) or F16 (0, kind::f16), K-major, N >> 3
// at bits 17-22, M = 256 (bits 24-28: M >> 4); the tile width n is a run-time value
template <int MODE>
__device__ __forceinline__ uint32_t idesc_pair(int n) {
    constexpr uint32_t f = MODE == MODE_TF32 ? 2u : 0u;
    return (1u << 4) | (f << 7) | (f << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(256 >> 4) << 24);
}
template <int MODE>
__device__ __forceinline__ void mma_pair(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
    if constexpr (MODE == MODE_TF32)
        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
                     "l"(a), "l"(b), "r"(idesc), "r"(acc));
    else
        asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
                     "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void commit_pair_multicast(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.multicast::cluster.b64 [%0], %1;" ::"r"(su32(bar)),
        "h"((uint16_t)3)
        : "memory");
}
__device__ __forceinline__ void commit_pair(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar)) : "memory");
}

// Output tile t -> (row block m, column block n) in bands of `group` row blocks, the row
// block fastest within a band: the tiles in flight at once (consecutive t over all CTAs)
// share a few B column blocks and a few A row blocks, so both stay in L2.
__device__ __forceinline__ void tile_mn(int t, int m_tiles, int n_tiles, int group, int& m, int& n) {
    const int band = t / (group * n_tiles), r = t - band * group * n_tiles;
    const int gm = min(group, m_tiles - band * group);
    n = r / gm;
    m = band * group + (r - n * gm);
}

template <int BN>
struct PairCfg {
    static constexpr int TILE_A = BM * 128;        // this CTA's 128 rows of A, 32 FP32 of K
    static constexpr int TILE_B = (BN / 2) * 128;  // this CTA's half of the BN rows of B
    static constexpr int STAGE = TILE_A + TILE_B;
    static constexpr int STAGES = SMEM_BUDGET / STAGE > 8 ? 8 : SMEM_BUDGET / STAGE;
    static_assert(STAGES >= 2, "stage ring too small");
};

// C[m, n] = sum_k A[m, k] B[n, k] over m_tiles (of 256 rows) x n_tiles output tiles of BN
// columns; the last tile of a row block is N - (n_tiles - 1) BN wide (a multiple of 32):
// each CTA still loads BN / 2 rows of B (rows past N read as zero) and the MMA takes the
// first width / 2 of them.
template <int MODE, int EPI, int BN>
__global__ void __launch_bounds__(THREADS, 1)
    k_tc_gemm_pair(const __grid_constant__ CUtensorMap tA, const __grid_constant__ CUtensorMap tB, int m_tiles, int n_tiles,
                   int group, int N, int kchunks, EpiParams ep, int* err) {
    using C = PairCfg<BN>;
    constexpr int S = C::STAGES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    float* epi_stage = reinterpret_cast<float*>(smem + (size_t)S * C::STAGE);  // 4 epilogue warps x 4 KB
    __shared__ __align__(8) uint64_t full[S], empty[S], tfull[2], tempty[2], drain;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t rank = cluster_rank();
    const bool leader = rank == 0;
    const int pair = blockIdx.x >> 1, npairs = gridDim.x >> 1;
    const int ntiles = m_tiles * n_tiles;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        for (int b = 0; b < 2; ++b) { mbar_init(&tfull[b], 1); mbar_init(&tempty[b], 8); }
        mbar_init(&drain, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {  // one warp of each CTA: the pair's TMEM, the same columns in both
        asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base)),
                     "r"(TMEM_COLS));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;");
    }
    fence_before();
    cluster_sync_all();  // barriers of both CTAs initialised before any cross-CTA signal
    fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer (both CTAs)
        // L2 policy by tile order: in bands (group > 1) a row block of A is reused by every
        // column block of its band, so it is kept like B; in the column-fastest order it is
        // used only while its tiles are in flight
        const uint64_t pol_a = group > 1 ? policy_evict_last() : policy_evict_first(), pol_b = policy_evict_last();
        int it = 0;
        bool ok = true;
        for (int tile = pair; tile < ntiles && ok; tile += npairs) {
            int mt, nt;
            tile_mn(tile, m_tiles, n_tiles, group, mt, nt);
            const int m0 = mt * (2 * BM) + (int)rank * BM;
            const int nb = nt * BN, width = min(BN, N - nb);
            const int n0 = nb + (int)rank * (width / 2);
            for (int kc = 0; kc < kchunks; ++kc, ++it) {
                const int s = it % S;
                if (it >= S && !mbar_wait(&empty[s], ((it / S) - 1) & 1, &abort_flag, err, 1)) { ok = false; break; }
                unsigned char* st = smem + (size_t)s * C::STAGE;
                const uint32_t fb = mapa_rank(su32(&full[s]), 0);
                if (leader) mbar_expect_tx(&full[s], 2 * C::STAGE);
                const int kx = kc * (MODE == MODE_TF32 ? 32 : 64);  // 128 bytes of K per stage
                tma_load_pair(st, &tA, kx, m0, fb, pol_a);
                tma_load_pair(st + C::TILE_A, &tB, kx, n0, fb, pol_b);
            }
        }
        if (!ok) {  // let the loads already issued land before the CTA exits
            for (int j = it - 1; j >= 0 && j >= it - S; --j) {
                if (leader) mbar_wait(&full[j % S], (j / S) & 1, &abort_flag, err, 0);
                else mbar_wait(&empty[j % S], (j / S) & 1, &abort_flag, err, 0);
            }
        }
    } else if (warp == 1 && lane == 0 && leader) {
        // ---------------- MMA issuer (leader CTA)
        int it = 0, t = 0;
        bool ok = true;
        for (int tile = pair; tile < ntiles && ok; tile += npairs, ++t) {
            const int buf = t & 1;
            if (t >= 2 && !mbar_wait(&tempty[buf], ((t >> 1) - 1) & 1, &abort_flag, err, 2)) break;
            fence_after();
            const uint32_t acc_addr = tmem + buf * ACC_STRIDE;
            int mt, nt;
            tile_mn(tile, m_tiles, n_tiles, group, mt, nt);
            const uint32_t id = idesc_pair<MODE>(min(BN, N - nt * BN));
            for (int kc = 0; kc < kchunks; ++kc, ++it) {
                const int s = it % S;
                if (!mbar_wait(&full[s], (it / S) & 1, &abort_flag, err, 2)) { ok = false; break; }
                fence_after();
                const uint32_t base = su32(smem + (size_t)s * C::STAGE);
                const uint32_t bbase = base + C::TILE_A;
#pragma unroll
                for (int kk = 0; kk < 4; ++kk) {
                    const uint32_t koff = kk * 32;  // 32 bytes (8 TF32 or 16 FP16) of K per instruction
                    mma_pair<MODE>(acc_addr, sdesc(base + koff), sdesc(bbase + koff), id, (kc > 0 || kk > 0) ? 1u : 0u);
                }
                commit_pair_multicast(&empty[s]);
            }
            if (ok) commit_pair_multicast(&tfull[buf]);
        }
        commit_pair(&drain);  // arrives once every MMA issued above has completed
        mbar_wait(&drain, 0, &abort_flag, err, 0);
    } else if (warp >= 2) {
        // ---------------- epilogue (both CTAs; warps 2-5, TMEM lane quarter = warp % 4)
        const int q = warp & 3;
        const uint32_t te0 = mapa_rank(su32(&tempty[0]), 0), te1 = mapa_rank(su32(&tempty[1]), 0);
        int t = 0;
        for (int tile = pair; tile < ntiles; tile += npairs, ++t) {
            const int buf = t & 1;
            int mt, nt;
            tile_mn(tile, m_tiles, n_tiles, group, mt, nt);
            const int m0 = mt * (2 * BM) + (int)rank * BM, n0 = nt * BN;
            const int width = min(BN, N - n0);
            if (!mbar_wait(&tfull[buf], (t >> 1) & 1, &abort_flag, err, 4)) break;
            fence_after();
            const int row = m0 + q * 32 + lane;
            float e_acc = 0.f;
#pragma unroll 1
            for (int cc = 0; cc < width / 32; ++cc) {
                float v[32];
                tmem_ld32(tmem + ((uint32_t)(q * 32) << 16) + buf * ACC_STRIDE + cc * 32, v);
                epilogue_chunk_staged<EPI>(ep, m0 + q * 32, lane, n0 + cc * 32, v, e_acc, epi_stage + q * 1024);
                if constexpr (EPI == EPI_KERNEL) {
                    if (cc & 1) {
                        if (row < ep.rows) ep.epart[(size_t)((n0 + cc * 32) / 64) * ep.rows + row] = (double)e_acc;
                        e_acc = 0.f;
                    }
                }
            }
            fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive_cluster(buf ? te1 : te0);
        }
    }
    fence_before();
    cluster_sync_all();  // no CTA leaves while its pair may still read its shared memory or TMEM
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS));
    }
}

__global__ void k_split_q(size_t n, const float* __restrict__ q, __nv_bfloat16* __restrict__ hi, __nv_bfloat16* __restrict__ lo) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = q[i];
    __nv_bfloat16 h = __float2bfloat16_rn(x);
    hi[i] = h;
    lo[i] = __float2bfloat16_rn(x - __bfloat162float(h));
}
__global__ void k_to_half(size_t n, const float* __restrict__ in, __half* __restrict__ out) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = __float2half_rn(in[i]);
}
// Energy of each centre from its per-block partials ([block][row]): four lanes per row,
// lane k summing blocks k, k + 4, ... in order, combined by an xor butterfly (fixed order).
__global__ void k_rowsum_scatter32(int nc, int ntiles, const double* __restrict__ epart, const int* __restrict__ centres,
                                   double* __restrict__ ecent, double* __restrict__ eatom) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x, i = g >> 2, sub = g & 3;
    double s = 0;
    if (i < nc)
        for (int t = sub; t < ntiles; t += 4) s += epart[(size_t)t * nc + i];
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    s += __shfl_xor_sync(0xffffffffu, s, 2);
    if (i >= nc || sub != 0) return;
    if (ecent) ecent[i] = s;  // per-centre energies (energy_per_coordinate)
    eatom[centres[i]] += s;
}

// ---------------------------------------------------------------- host helpers
uint16_t host_bf16(float f) {  // round to nearest even
    uint32_t b;
    std::memcpy(&b, &f, 4);
    if ((b & 0x7f800000u) == 0x7f800000u) return (uint16_t)(b >> 16);
    b += 0x7fffu + ((b >> 16) & 1u);
    return (uint16_t)(b >> 16);
}
float bf16_to_f(uint16_t h) {
    uint32_t b = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &b, 4);
    return f;
}
float host_tf32(float f) {  // round to nearest, ties away (cvt.rna)
    uint32_t b;
    std::memcpy(&b, &f, 4);
    if ((b & 0x7f800000u) != 0x7f800000u) { b += 0x1000u; b &= 0xffffe000u; }
    float r;
    std::memcpy(&r, &b, 4);
    return r;
}

// The driver's tensor-map encoder, resolved through the runtime so that the library
// does not link libcuda directly.
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

int make_map(CUtensorMap* tm, void* base, CUtensorMapDataType dt, int esize, uint64_t inner, uint64_t outer, uint32_t box_inner,
             uint32_t box_outer = BM) {
    auto enc = encode_fn();
    if (!enc) GG_FAIL(GAPGPU_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * (cuuint64_t)esize};
    cuuint32_t box[2] = {box_inner, box_outer};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(tm, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) GG_FAIL(GAPGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GAPGPU_OK;
}

int num_sms() {
    static int n[64] = {0};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= 64) return 148;
    if (!n[dev]) cudaDeviceGetAttribute(&n[dev], cudaDevAttrMultiProcessorCount, dev);
    return n[dev] > 0 ? n[dev] : 148;
}

// Widest N tile that divides N (operands are padded to multiples of 128).
int pick_bn(int MODE, int N) {
    if (MODE == MODE_BF16X3) return 128;  // two hi/lo planes per operand: wider tiles leave < 3 stages
    if (N % 256 == 0) return 256;
    if (N % 192 == 0) return 192;
    return 128;
}

// ---------------------------------------------------------------- autotuner
// The first GEMM of a shape (mode, epilogue, N, K, log2 of the row count) times every
// N tile that divides N and leaves at least two pipeline stages, on the real operands
// (each candidate rewrites the same outputs), and keeps the fastest for the process --
// the timing loop of IP_setup_parallel (src/Potentials/IP.f95:1092-1134) applied to
// tile shapes.  Inside a stream capture no timing is possible: the heuristic decides.
struct TuneKey {
    int mode, epi, N, K, rb, pairs, wf16;
    bool operator<(const TuneKey& o) const {
        return std::tie(mode, epi, N, K, rb, pairs, wf16) < std::tie(o.mode, o.epi, o.N, o.K, o.rb, o.pairs, o.wf16);
    }
};
// A tile choice: BN > 0 one CTA per 128-row tile, BN < 0 a CTA pair per 256-row tile of -BN columns.
struct TuneEntry {
    int bn;
    std::vector<std::pair<int, float>> timings;  // (tile choice, ms)
};
std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;
std::map<TuneKey, int> g_rule;  // shapes whose tile the built-in rule chose (reported, never tuned from)

int rows_bucket(int rows) {
    int b = 0;
    while ((1 << b) < rows && b < 30) ++b;
    return b;
}

// pairs: 0 single-CTA tiles only, 1 also CTA-pair tiles (TF32), 2 CTA-pair tiles only
template <int MODE>
std::vector<int> bn_candidates(int N, int pairs) {
    std::vector<int> c;
    if (MODE == MODE_F16) pairs = 2;  // FP16 tiles exist on CTA pairs only
    else if (MODE != MODE_TF32) pairs = 0;
    if (pairs < 2) {
        if (N % 256 == 0 && Cfg<MODE, 256>::STAGES >= 2) c.push_back(256);
        if (N % 192 == 0 && Cfg<MODE, 192>::STAGES >= 2) c.push_back(192);
        c.push_back(128);
    }
    if (pairs >= 1) {  // N is a multiple of 128: 256-wide pair tiles end in a 128-wide one
        if (N >= 256) c.push_back(-256);
        if (N % 192 == 0) c.push_back(-192);
        c.push_back(-128);
    }
    return c;
}

// Row blocks per band of the pair kernels' tile order: bands of 16 when there are many
// column blocks (the sparse-point operand B is then the one shared by the tiles in
// flight), none when there are few (the row blocks of A are then the large operand, and
// the N-fastest order keeps each one in L2 until all its column blocks are done).
int pair_tile_group(int n_tiles) { return n_tiles >= 16 ? 16 : 1; }

template <int MODE, int EPI, int BN>
int launch_pair(gapgpu_context& c, const CUtensorMap& a, const CUtensorMap& b, int rows, int N, int kchunks, EpiParams ep,
                int* err) {
    using Cf = PairCfg<BN>;
    const int smem = Cf::STAGES * Cf::STAGE + 4 * 4096 + 1024;  // stage ring, epilogue stages, alignment
    GG_CUDA(cudaFuncSetAttribute(k_tc_gemm_pair<MODE, EPI, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int m_tiles = (rows + 2 * BM - 1) / (2 * BM), n_tiles = (N + BN - 1) / BN;
    if (EPI == EPI_KERNEL) ep.ntiles = N / 64;  // energy blocks of 64 columns
    const int ntiles = m_tiles * n_tiles;
    cudaLaunchConfig_t cfg = {};
    cfg.blockDim = dim3(THREADS);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = c.stream;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = 2;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    // persistent: as many pairs as can be resident at once (clusters stay within a GPC)
    cfg.gridDim = dim3(2 * (num_sms() / 2));
    int resident = 0;
    GG_CUDA(cudaOccupancyMaxActiveClusters(&resident, k_tc_gemm_pair<MODE, EPI, BN>, &cfg));
    const int npairs = std::max(1, std::min(ntiles, resident > 0 ? resident : num_sms() / 2));
    cfg.gridDim = dim3(2 * npairs);
    GG_CUDA(cudaLaunchKernelEx(&cfg, k_tc_gemm_pair<MODE, EPI, BN>, a, b, m_tiles, n_tiles, pair_tile_group(n_tiles), N, kchunks, ep,
                               err));
    c.launches++;
    return GAPGPU_OK;
}

template <int MODE, int EPI, int BN>
int launch_bn(gapgpu_context& c, const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b0,
              const CUtensorMap& b1, int rows, int N, int kchunks, EpiParams ep, int* err) {
    using Cf = Cfg<MODE, BN>;
    const int smem = Cf::STAGES * Cf::STAGE + 1024;
    GG_CUDA(cudaFuncSetAttribute(k_tc_gemm<MODE, EPI, BN>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const int m_tiles = (rows + BM - 1) / BM, n_tiles = N / BN;
    if (EPI == EPI_KERNEL) ep.ntiles = N / 64;  // energy blocks of 64 columns
    const int ntiles = m_tiles * n_tiles;
    const int grid = std::min(ntiles, num_sms());
    k_tc_gemm<MODE, EPI, BN><<<grid, THREADS, smem, c.stream>>>(a0, a1, b0, b1, m_tiles, n_tiles, kchunks, ep, err);
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

// One GEMM C = A B^T with the operand maps built here: A [rows x K] (planes a0, a1),
// B [N x K] (planes b0, b1), both K-contiguous.
template <int MODE, int EPI>
int launch_any(gapgpu_context& c, int BN, const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b0,
               const CUtensorMap& b1, int rows, int N, int kchunks, const EpiParams& ep, int* err) {
    if constexpr (MODE == MODE_TF32 || MODE == MODE_F16) {
        if (BN == -256) return launch_pair<MODE, EPI, 256>(c, a0, b0, rows, N, kchunks, ep, err);
        if (BN == -192) return launch_pair<MODE, EPI, 192>(c, a0, b0, rows, N, kchunks, ep, err);
        if (BN == -128 || MODE == MODE_F16) return launch_pair<MODE, EPI, 128>(c, a0, b0, rows, N, kchunks, ep, err);
    }
    if constexpr (MODE == MODE_F16) {
        GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "FP16 GEMMs run on CTA pairs only");
    } else {
        if (BN == 256) return launch_bn<MODE, EPI, 256>(c, a0, a1, b0, b1, rows, N, kchunks, ep, err);
        if (BN == 192) return launch_bn<MODE, EPI, 192>(c, a0, a1, b0, b1, rows, N, kchunks, ep, err);
        return launch_bn<MODE, EPI, 128>(c, a0, a1, b0, b1, rows, N, kchunks, ep, err);
    }
}

// One GEMM C = A B^T with the operand maps built here: A [rows x K] (planes a0, a1),
// B [N x K] (planes b0, b1), both K-contiguous.
template <int MODE, int EPI>
int gemm(gapgpu_context& c, void* a0p, void* a1p, void* b0p, void* b1p, int rows, int N, int K, EpiParams ep, int* err,
         int* ntiles_out) {
    const CUtensorMapDataType dt = MODE == MODE_BF16X3 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16
                                   : MODE == MODE_F16  ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                       : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    const int es = MODE == MODE_TF32 ? 4 : 2, KB = 128 / es;
    const int kchunks = K / KB;
    int rc;
    auto maps = [&](int BN, CUtensorMap& a0, CUtensorMap& a1, CUtensorMap& b0, CUtensorMap& b1) {
        int r;
        // a CTA pair loads half of the B tile in each CTA
        const uint32_t bbox = BN > 0 ? (uint32_t)BN : (uint32_t)(-BN / 2);
        if ((r = make_map(&a0, a0p, dt, es, K, rows, KB)) || (r = make_map(&b0, b0p, dt, es, K, N, KB, bbox))) return r;
        if (MODE == MODE_BF16X3) {
            if ((r = make_map(&a1, a1p, dt, es, K, rows, KB)) || (r = make_map(&b1, b1p, dt, es, K, N, KB, bbox))) return r;
        } else {
            a1 = a0;
            b1 = b0;
        }
        return (int)GAPGPU_OK;
    };
    const int pairs = MODE == MODE_TF32 ? c.gemm_pairs : MODE == MODE_F16 ? 2 : 0;
    const TuneKey key{MODE, EPI, N, K, rows_bucket(rows), pairs, ep.w_f16};
    int BN = 0;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto it = g_tune.find(key);
        if (it != g_tune.end()) BN = it->second.bn;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    GG_CUDA(cudaStreamIsCapturing(c.stream, &cap));
    if (!BN && c.autotune && cap == cudaStreamCaptureStatusNone) {
        TuneEntry te{0, {}};
        cudaEvent_t e0, e1;
        GG_CUDA(cudaEventCreate(&e0));
        GG_CUDA(cudaEventCreate(&e1));
        float best = 1e30f;
        for (int bn : bn_candidates<MODE>(N, pairs)) {
            CUtensorMap a0, a1, b0, b1;
            if ((rc = maps(bn, a0, a1, b0, b1))) return rc;
            if ((rc = launch_any<MODE, EPI>(c, bn, a0, a1, b0, b1, rows, N, kchunks, ep, err))) return rc;  // warm
            GG_CUDA(cudaEventRecord(e0, c.stream));
            if ((rc = launch_any<MODE, EPI>(c, bn, a0, a1, b0, b1, rows, N, kchunks, ep, err))) return rc;
            GG_CUDA(cudaEventRecord(e1, c.stream));
            GG_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            te.timings.push_back({bn, ms});
            if (ms < best) { best = ms; te.bn = bn; }
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        BN = te.bn;
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = te;
    }
    // without a timing (inside a capture, or autotuning off): 256-wide pair tiles where
    // enabled -- the fastest candidate at every row count measured on GB300
    if (!BN) {
        BN = pairs >= 1 ? (N >= 256 ? -256 : -128) : pick_bn(MODE, N);
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_rule[key] = BN;
    }
    CUtensorMap a0, a1, b0, b1;
    if ((rc = maps(BN, a0, a1, b0, b1))) return rc;
    if (ntiles_out) *ntiles_out = N / 64;
    return launch_any<MODE, EPI>(c, BN, a0, a1, b0, b1, rows, N, kchunks, ep, err);
}

template <int MODE>
int run_mixed(gapgpu_context& c, const Coordinate& co, int nc) {
    const int Dp = co.Dpad, Mp = co.Mpad;
    const size_t nq = (size_t)nc * Dp, nw = (size_t)nc * Mp;
    int rc;
    const size_t es = MODE == MODE_BF16X3 ? 2 : 4;
    const int ntiles_max = Mp / 64;
    if ((rc = c.Kbuf.ensure(es * nq)) || (rc = c.qlo.ensure(es * nq)) || (rc = c.Wbuf.ensure(es * nw)) ||
        (rc = c.Wlo.ensure(es * nw)) || (rc = c.epart.ensure(sizeof(double) * (size_t)nc * ntiles_max)) ||
        (rc = c.Gbuf.ensure(sizeof(float) * nq)) || (rc = c.total.ensure(sizeof(int) * 4)))
        return rc;
    int* err = c.total.as<int>() + 3;  // cleared at the start of the evaluation, read after it
    const int TB = 256;
    const unsigned nb = (unsigned)((nq + TB - 1) / TB);
    // TF32: the forward kernel wrote the rounded descriptors to qlo next to q
    if (MODE == MODE_BF16X3) {
        k_split_q<<<nb, TB, 0, c.stream>>>(nq, c.qbuf.as<float>(), c.Kbuf.as<__nv_bfloat16>(), c.qlo.as<__nv_bfloat16>());
        c.launches++;
    }
    const double z = co.zeta;
    // TF32 with CTA pairs: the second GEMM in FP16 when the model's operands allow it --
    // the first GEMM's epilogue writes W' = S K^(zeta-1) in FP16 and the sparse points carry
    // coef zeta / S (both 10-bit mantissas, like TF32; half the W bytes, twice the MMA rate)
    const bool f16 = MODE == MODE_TF32 && c.gemm2_f16 && c.gemm_pairs >= 1 && co.dXTh16 != nullptr;
    EpiParams ep{nc, Mp, co.dcoef32, (float)z, (z == std::floor(z) && z >= 1 && z <= 64) ? (int)z : 0, c.Wbuf.p, c.Wlo.p,
                 c.epart.as<double>(), 0, f16 ? 1 : 0, (float)co.f16_scale};
    int ntiles = 0;
    // GEMM1: K = Q X^T with the kernel epilogue (W and per-tile energies); in FP16 when the
    // forward kernel wrote the descriptors in FP16
    if (MODE == MODE_BF16X3)
        rc = gemm<MODE, EPI_KERNEL>(c, c.Kbuf.p, c.qlo.p, co.dXhi, co.dXlo, nc, Mp, Dp, ep, err, &ntiles);
    else if (gemm1_f16_active(c, co))
        rc = gemm<MODE_F16, EPI_KERNEL>(c, c.qlo.p, c.qlo.p, co.dXh16, co.dXh16, nc, Mp, Dp, ep, err, &ntiles);
    else
        rc = gemm<MODE, EPI_KERNEL>(c, c.qlo.p, c.qlo.p, co.dXf32, co.dXf32, nc, Mp, Dp, ep, err, &ntiles);
    if (rc) return rc;
    if (c.want_epc && (rc = c.ecent.ensure(sizeof(double) * (size_t)nc))) return rc;
    k_rowsum_scatter32<<<(unsigned)((4 * (size_t)nc + 127) / 128), 128, 0, c.stream>>>(nc, ntiles, c.epart.as<double>(), c.cur_centres,
                                                              c.want_epc ? c.ecent.as<double>() : nullptr,
                                                              c.eatom.as<double>());
    c.launches++;
    // GEMM2: G = W X, B operand = X^T rows (k = sparse index contiguous)
    EpiParams ep2{nc, Dp, nullptr, 0.f, 0, c.Gbuf.p, nullptr, nullptr, 0, 0, 0.f};
    if (MODE == MODE_BF16X3)
        rc = gemm<MODE, EPI_STORE>(c, c.Wbuf.p, c.Wlo.p, co.dXThi, co.dXTlo, nc, Dp, Mp, ep2, err, nullptr);
    else if (f16)
        rc = gemm<MODE_F16, EPI_STORE>(c, c.Wbuf.p, c.Wbuf.p, co.dXTh16, co.dXTh16, nc, Dp, Mp, ep2, err, nullptr);
    else
        rc = gemm<MODE, EPI_STORE>(c, c.Wbuf.p, c.Wbuf.p, co.dXTf32, co.dXTf32, nc, Dp, Mp, ep2, err, nullptr);
    return rc;
}

}  // namespace

// Model-level operands for the mixed path (host-side conversion, FP64 source).
int prepare_mixed_operands(gapgpu_model& m) {
    for (Coordinate& co : m.coords) {
        if (co.type == DESC_DISTANCE_2B) {  // FP32 sparse points and coefficients of the mixed pair kernel
            std::vector<float> x(co.M), cf(co.M);
            for (int s = 0; s < co.M; ++s) {
                x[s] = (float)co.X[s];
                cf[s] = (float)(co.alpha[s] * co.sc[s] * co.delta * co.delta);
            }
            GG_CUDA(cudaMalloc(&co.dXf32, sizeof(float) * std::max(co.M, 1)));
            GG_CUDA(cudaMalloc(&co.dcoef32, sizeof(float) * std::max(co.M, 1)));
            if (co.M > 0) {
                GG_CUDA(cudaMemcpy(co.dXf32, x.data(), sizeof(float) * co.M, cudaMemcpyHostToDevice));
                GG_CUDA(cudaMemcpy(co.dcoef32, cf.data(), sizeof(float) * co.M, cudaMemcpyHostToDevice));
            }
            continue;
        }
        if (co.type != DESC_SOAP) continue;
        const int Dp = co.Dpad, Mp = co.Mpad;
        const size_t ne = (size_t)Mp * Dp;
        std::vector<float> xf(ne, 0.f), xtf(ne, 0.f), coef(Mp, 0.f);
        std::vector<uint16_t> xh(ne, 0), xl(ne, 0), xth(ne, 0), xtl(ne, 0);
        for (int s = 0; s < co.M; ++s) {
            coef[s] = (float)(co.alpha[s] * co.sc[s] * co.delta * co.delta);
            for (int d = 0; d < co.D; ++d) {
                double x = co.X[(size_t)s * co.D + d];
                float t = host_tf32((float)x);
                uint16_t h = host_bf16((float)x);
                uint16_t l = host_bf16((float)(x - (double)bf16_to_f(h)));
                size_t a = (size_t)s * Dp + d, b = (size_t)d * Mp + s;
                xf[a] = t; xtf[b] = t;
                xh[a] = h; xl[a] = l; xth[b] = h; xtl[b] = l;
            }
        }
        GG_CUDA(cudaMalloc(&co.dXf32, sizeof(float) * ne));
        GG_CUDA(cudaMalloc(&co.dXTf32, sizeof(float) * ne));
        GG_CUDA(cudaMalloc(&co.dXhi, 2 * ne));
        GG_CUDA(cudaMalloc(&co.dXlo, 2 * ne));
        GG_CUDA(cudaMalloc(&co.dXThi, 2 * ne));
        GG_CUDA(cudaMalloc(&co.dXTlo, 2 * ne));
        GG_CUDA(cudaMalloc(&co.dcoef32, sizeof(float) * Mp));
        GG_CUDA(cudaMemcpy(co.dXf32, xf.data(), sizeof(float) * ne, cudaMemcpyHostToDevice));
        GG_CUDA(cudaMemcpy(co.dXTf32, xtf.data(), sizeof(float) * ne, cudaMemcpyHostToDevice));
        GG_CUDA(cudaMemcpy(co.dXhi, xh.data(), 2 * ne, cudaMemcpyHostToDevice));
        GG_CUDA(cudaMemcpy(co.dXlo, xl.data(), 2 * ne, cudaMemcpyHostToDevice));
        GG_CUDA(cudaMemcpy(co.dXThi, xth.data(), 2 * ne, cudaMemcpyHostToDevice));
        GG_CUDA(cudaMemcpy(co.dXTlo, xtl.data(), 2 * ne, cudaMemcpyHostToDevice));
        GG_CUDA(cudaMemcpy(co.dcoef32, coef.data(), sizeof(float) * Mp, cudaMemcpyHostToDevice));
        // FP16 sparse points of the FP16 second GEMM: X'[d][m] = (coef_m zeta / S) x_m[d] with
        // S = max_m |coef_m zeta|, paired with W' = S K^(zeta-1) written by the first GEMM.  Only
        // for integer zeta and normalised descriptors, and when S kmax^(zeta-1) stays far below
        // the FP16 maximum (kmax: the largest possible |q.x|); otherwise the second GEMM is TF32.
        co.f16_scale = 0.0;
        const double zt = co.zeta;
        double S = 0.0, xn = 0.0;
        for (int s = 0; s < co.M; ++s) {
            S = std::max(S, std::fabs(co.alpha[s] * co.sc[s] * co.delta * co.delta * zt));
            double n2 = 0.0;
            for (int d = 0; d < co.D; ++d) n2 += co.X[(size_t)s * co.D + d] * co.X[(size_t)s * co.D + d];
            xn = std::max(xn, std::sqrt(n2));
        }
        const double kmax = std::sqrt(1.0 + co.soap.sigma0 * co.soap.sigma0) * xn;
        if (zt == std::floor(zt) && zt >= 1 && zt <= 64 && co.soap.normalise && S > 0 &&
            S * std::pow(std::max(kmax, 1.0), zt - 1) <= 1e4) {
            std::vector<float> xs(ne, 0.f);
            for (int s = 0; s < co.M; ++s) {
                const double f = co.alpha[s] * co.sc[s] * co.delta * co.delta * zt / S;
                for (int d = 0; d < co.D; ++d) xs[(size_t)d * Mp + s] = (float)(f * co.X[(size_t)s * co.D + d]);
            }
            // and the unscaled sparse points of the FP16 first GEMM (normalised vectors: |x| <= xn)
            std::vector<float> xr(ne, 0.f);
            for (int s = 0; s < co.M; ++s)
                for (int d = 0; d < co.D; ++d) xr[(size_t)s * Dp + d] = (float)co.X[(size_t)s * co.D + d];
            float* tmp = nullptr;
            GG_CUDA(cudaMalloc(&tmp, sizeof(float) * ne));
            GG_CUDA(cudaMalloc(&co.dXTh16, 2 * ne));
            GG_CUDA(cudaMalloc(&co.dXh16, 2 * ne));
            GG_CUDA(cudaMemcpy(tmp, xs.data(), sizeof(float) * ne, cudaMemcpyHostToDevice));
            k_to_half<<<(unsigned)((ne + 255) / 256), 256>>>(ne, tmp, reinterpret_cast<__half*>(co.dXTh16));
            cudaError_t e = cudaDeviceSynchronize();
            if (e == cudaSuccess) e = cudaMemcpy(tmp, xr.data(), sizeof(float) * ne, cudaMemcpyHostToDevice);
            if (e == cudaSuccess) {
                k_to_half<<<(unsigned)((ne + 255) / 256), 256>>>(ne, tmp, reinterpret_cast<__half*>(co.dXh16));
                e = cudaDeviceSynchronize();
            }
            cudaFree(tmp);
            if (e != cudaSuccess) GG_FAIL(GAPGPU_ERR_CUDA, std::string("FP16 operands: ") + cudaGetErrorString(e));
            co.f16_scale = S;
        }
    }
    return GAPGPU_OK;
}

int gp_mixed(gapgpu_context& c, const Coordinate& co, int nc, int precision) {
    if (nc == 0) return GAPGPU_OK;
    if (co.cov != COV_DOT_PRODUCT) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "SOAP coordinates need the dot_product covariance");
    if (co.Dpad % 128 || co.Mpad % 128) GG_FAIL(GAPGPU_ERR_ARG, "internal: operand padding is not a multiple of 128");
    return precision == GAPGPU_MIXED_BF16X3 ? run_mixed<MODE_BF16X3>(c, co, nc) : run_mixed<MODE_TF32>(c, co, nc);
}

}  // namespace gapgpu

namespace {
std::string tile_name(int bn) { return bn > 0 ? std::to_string(bn) : "2x" + std::to_string(-bn); }
}  // namespace

extern "C" int gapgpu_tuning_report(char* buf, int capacity) {
    using namespace gapgpu;
    std::string out;
    std::lock_guard<std::mutex> lk(g_tune_mu);
    for (const auto& kv : g_tune) {
        const TuneKey& k = kv.first;
        out += std::string(k.mode == MODE_BF16X3 ? "bf16x3" : k.mode == MODE_F16 ? "f16" : "tf32") +
               (k.epi == EPI_KERNEL ? (k.wf16 ? " kernel->f16" : " kernel") : " store") +
               " N=" + std::to_string(k.N) + " K=" + std::to_string(k.K) + " rows<=2^" + std::to_string(k.rb) +
               " BN=" + tile_name(kv.second.bn) + " [";
        for (size_t i = 0; i < kv.second.timings.size(); ++i) {
            char t[64];
            std::snprintf(t, sizeof t, "%s%s:%.3fms", i ? " " : "", tile_name(kv.second.timings[i].first).c_str(),
                          kv.second.timings[i].second);
            out += t;
        }
        out += "]\n";
    }
    for (const auto& kv : g_rule) {
        const TuneKey& k = kv.first;
        if (g_tune.count(k)) continue;
        out += std::string(k.mode == MODE_BF16X3 ? "bf16x3" : k.mode == MODE_F16 ? "f16" : "tf32") +
               (k.epi == EPI_KERNEL ? (k.wf16 ? " kernel->f16" : " kernel") : " store") + " N=" + std::to_string(k.N) +
               " K=" + std::to_string(k.K) + " rows<=2^" + std::to_string(k.rb) + " BN=" + tile_name(kv.second) +
               " [rule]\n";
    }
    if (buf && capacity > 0) {
        std::strncpy(buf, out.c_str(), (size_t)capacity - 1);
        buf[capacity - 1] = 0;
    }
    return (int)out.size();
}

extern "C" int gapgpu_selftest_bounded_wait(gapgpu_context* c, int64_t limit_us) {
    using namespace gapgpu;
    if (!c || limit_us < 1 || limit_us > 1000000) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_selftest_bounded_wait: bad argument");
    int rc;
    if ((rc = c->total.ensure(sizeof(int) * 4))) return rc;
    int* err = c->total.as<int>() + 3;
    GG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c->stream));
    k_wait_probe<<<1, 32, 0, c->stream>>>(1000ull * (unsigned long long)limit_us, err);
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaStreamSynchronize(c->stream));
    return check_device_flags(*c);
}
