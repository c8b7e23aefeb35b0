// tcgen05.cu -- K5 mixed path: the sparse-GP kernel GEMMs on Blackwell tensor cores.
//
//   GEMM1  K = Q X^T   [nc x M]  fused epilogue: W = coef zeta K^(zeta-1) and per-tile
//                                 row sums of coef K^zeta (the local energies)
//   GEMM2  G = W X     [nc x D]  (dE/dq of every centre)
// Two operand encodings, both with FP32 accumulation in TMEM:
//   bf16x3: every operand is split x = hi + lo (bf16 each) and the product is
//           hi*hi + hi*lo + lo*hi (three tcgen05.mma kind::f16 per k-step; the dropped
//           lo*lo term is 2^-16 relative);
//   tf32:   operands rounded to TF32 (cvt.rna), one tcgen05.mma kind::tf32 per k-step.
// Structure of one CTA (128 threads, one 128x128 output tile):
//   warp 0 lane 0  TMA producer: 2-D tiled loads, 128B swizzle, into an S-stage ring
//   warp 1 lane 0  MMA issuer: tcgen05.mma from shared-memory descriptors into TMEM,
//                  tcgen05.commit frees each stage and finally signals the epilogue
//   warps 0-3      epilogue: tcgen05.ld 32x32b (warp w owns TMEM lanes 32w..32w+31)
// Every mbarrier wait is bounded; on expiry the kernel records an error code, waits
// (bounded) for its own work in flight, frees its TMEM and returns.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <cstring>
#include <cmath>
#include <vector>
#include <algorithm>

#include "context.h"

namespace gapgpu {
namespace {

constexpr int BM = 128, BN = 128, THREADS = 128;
constexpr int MODE_BF16X3 = 1, MODE_TF32 = 2;
constexpr int EPI_KERNEL = 1, EPI_STORE = 2;
constexpr long long WAIT_LIMIT = 1LL << 24;

template <int MODE> struct Cfg;
template <> struct Cfg<MODE_BF16X3> {
    static constexpr int KB = 64;              // k elements per stage (128 bytes)
    static constexpr int TILE_A = BM * 128;    // bytes of one A tile (hi or lo)
    static constexpr int TILE_B = BN * 128;
    static constexpr int STAGE = 2 * TILE_A + 2 * TILE_B;
    static constexpr int STAGES = 3;
    static constexpr int KSTEP = 16;           // k per tcgen05.mma
};
template <> struct Cfg<MODE_TF32> {
    static constexpr int KB = 32;
    static constexpr int TILE_A = BM * 128;
    static constexpr int TILE_B = BN * 128;
    static constexpr int STAGE = TILE_A + TILE_B;
    static constexpr int STAGES = 6;
    static constexpr int KSTEP = 8;
};

__device__ __forceinline__ uint32_t su32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, int count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(su32(b)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(su32(b)), "r"(bytes) : "memory");
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
// Bounded wait.  Gives up when the limit is reached or another thread of the CTA
// already gave up (abort flag in shared memory).
__device__ __forceinline__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, int* err, int code) {
    for (long long i = 0; i < WAIT_LIMIT; ++i) {
        if (mbar_try(b, parity)) return true;
        if ((i & 1023) == 1023 && *abort_flag) return false;
    }
    *abort_flag = 1;
    atomicOr(err, code);
    return false;
}

__device__ __forceinline__ void tma_load(void* dst, const CUtensorMap* tm, int c0, int c1, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            su32(dst)),
        "l"(reinterpret_cast<uint64_t>(tm)), "r"(c0), "r"(c1), "r"(su32(bar))
        : "memory");
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

template <int MODE>
__device__ __forceinline__ constexpr uint32_t idesc() {
    // D = F32 (bit 4); A/B format bits 7-9 / 10-12 (BF16 = 1 for kind::f16, TF32 = 2 for
    // kind::tf32); K-major A and B; N >> 3 at bits 17-22; M >> 4 at bits 24-28.
    return (1u << 4) | ((MODE == MODE_BF16X3 ? 1u : 2u) << 7) | ((MODE == MODE_BF16X3 ? 1u : 2u) << 10) |
           ((uint32_t)(BN >> 3) << 17) | ((uint32_t)(BM >> 4) << 24);
}

template <int MODE>
__device__ __forceinline__ void mma(uint32_t dt, uint64_t a, uint64_t b, uint32_t acc) {
    if constexpr (MODE == MODE_BF16X3)
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
            "l"(a), "l"(b), "r"(idesc<MODE>()), "r"(acc));
    else
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(dt),
            "l"(a), "l"(b), "r"(idesc<MODE>()), "r"(acc));
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

__device__ __forceinline__ float round_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}

struct EpiParams {
    int rows;             // valid rows (centres)
    int ldo;              // leading dimension of the outputs
    const float* coef;    // [N] alpha * sparseCutoff * delta^2   (EPI_KERNEL)
    float zeta;
    int izeta;
    void* out_hi;         // W (bf16 hi or tf32 fp32) / G (fp32)
    void* out_lo;         // W lo (bf16x3)
    double* epart;        // [rows x ntiles]
    int ntiles;
};

template <int MODE, int EPI>
__global__ void __launch_bounds__(THREADS, 1)
    k_tc_gemm(const __grid_constant__ CUtensorMap tA0, const __grid_constant__ CUtensorMap tA1,
              const __grid_constant__ CUtensorMap tB0, const __grid_constant__ CUtensorMap tB1, int kchunks, EpiParams ep,
              int* err) {
    using C = Cfg<MODE>;
    constexpr int S = C::STAGES;
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char* smem = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    __shared__ __align__(8) uint64_t full[S], empty[S], accum;
    __shared__ uint32_t tmem_base;
    __shared__ volatile int abort_flag;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    if (threadIdx.x == 0) {
        for (int s = 0; s < S; ++s) { mbar_init(&full[s], 1); mbar_init(&empty[s], 1); }
        mbar_init(&accum, 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_base)), "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_base;

    if (warp == 0 && lane == 0) {
        // ---------------- TMA producer
        for (int kc = 0; kc < kchunks; ++kc) {
            const int s = kc % S;
            if (kc >= S && !mbar_wait(&empty[s], ((kc / S) - 1) & 1, &abort_flag, err, 1)) break;
            unsigned char* st = smem + (size_t)s * C::STAGE;
            mbar_expect_tx(&full[s], C::STAGE);
            const int kx = kc * C::KB;
            if constexpr (MODE == MODE_BF16X3) {
                tma_load(st, &tA0, kx, m0, &full[s]);
                tma_load(st + C::TILE_A, &tA1, kx, m0, &full[s]);
                tma_load(st + 2 * C::TILE_A, &tB0, kx, n0, &full[s]);
                tma_load(st + 2 * C::TILE_A + C::TILE_B, &tB1, kx, n0, &full[s]);
            } else {
                tma_load(st, &tA0, kx, m0, &full[s]);
                tma_load(st + C::TILE_A, &tB0, kx, n0, &full[s]);
            }
        }
    } else if (warp == 1 && lane == 0) {
        // ---------------- MMA issuer
        bool ok = true;
        for (int kc = 0; kc < kchunks && ok; ++kc) {
            const int s = kc % S;
            if (!mbar_wait(&full[s], (kc / S) & 1, &abort_flag, err, 2)) { ok = false; break; }
            fence_after();
            const uint32_t base = su32(smem + (size_t)s * C::STAGE);
#pragma unroll
            for (int kk = 0; kk < C::KB / C::KSTEP; ++kk) {
                const uint32_t koff = kk * 32;  // 32 bytes of K per instruction
                const uint32_t acc = (kc > 0 || kk > 0) ? 1u : 0u;
                if constexpr (MODE == MODE_BF16X3) {
                    uint64_t ah = sdesc(base + koff), al = sdesc(base + C::TILE_A + koff);
                    uint64_t bh = sdesc(base + 2 * C::TILE_A + koff), bl = sdesc(base + 2 * C::TILE_A + C::TILE_B + koff);
                    mma<MODE>(tmem, ah, bh, acc);
                    mma<MODE>(tmem, ah, bl, 1u);
                    mma<MODE>(tmem, al, bh, 1u);
                } else {
                    uint64_t a = sdesc(base + koff), b = sdesc(base + C::TILE_A + koff);
                    mma<MODE>(tmem, a, b, acc);
                }
            }
            mma_commit(&empty[s]);
        }
        mma_commit(&accum);  // arrives once every MMA issued above has completed
    }
    __syncwarp();
    // ---------------- epilogue (all 4 warps)
    bool have = mbar_wait(&accum, 0, &abort_flag, err, 4);
    fence_after();
    const int row = m0 + warp * 32 + lane;
    // tcgen05.ld is warp-collective: decide per warp
    if (__all_sync(0xffffffffu, have && !abort_flag)) {
        float e_acc = 0.f;
#pragma unroll 1
        for (int cc = 0; cc < BN / 32; ++cc) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + cc * 32, v);
            const int col0 = n0 + cc * 32;
            if (row >= ep.rows) continue;
            if constexpr (EPI == EPI_KERNEL) {
                float w[32];
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    float k = v[j], cf = ep.coef[col0 + j];
                    float km1;
                    if (ep.izeta == 4) km1 = k * k * k;
                    else if (ep.izeta > 0) { km1 = 1.f; for (int t = 1; t < ep.izeta; ++t) km1 *= k; }
                    else km1 = powf(k, ep.zeta - 1.f);
                    e_acc += cf * km1 * k;
                    w[j] = cf * ep.zeta * km1;
                }
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
                        oh[q] = reinterpret_cast<const uint4*>(hi)[q];
                        ol[q] = reinterpret_cast<const uint4*>(lo)[q];
                    }
                } else {
                    float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(ep.out_hi) + (size_t)row * ep.ldo + col0);
#pragma unroll
                    for (int q = 0; q < 8; ++q)
                        o[q] = make_float4(round_tf32(w[4 * q]), round_tf32(w[4 * q + 1]), round_tf32(w[4 * q + 2]),
                                           round_tf32(w[4 * q + 3]));
                }
            } else {
                float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(ep.out_hi) + (size_t)row * ep.ldo + col0);
#pragma unroll
                for (int q = 0; q < 8; ++q) o[q] = make_float4(v[4 * q], v[4 * q + 1], v[4 * q + 2], v[4 * q + 3]);
            }
        }
        if constexpr (EPI == EPI_KERNEL) {
            if (row < ep.rows) ep.epart[(size_t)row * ep.ntiles + blockIdx.x] = (double)e_acc;
        }
    }
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
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
__global__ void k_round_q(size_t n, const float* __restrict__ q, float* __restrict__ out) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = round_tf32(q[i]);
}
__global__ void k_rowsum_scatter32(int nc, int ntiles, const double* __restrict__ epart, const int* __restrict__ centres,
                                   double* __restrict__ eatom) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double s = 0;
    for (int t = 0; t < ntiles; ++t) s += epart[(size_t)i * ntiles + t];
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

int make_map(CUtensorMap* tm, void* base, CUtensorMapDataType dt, int esize, uint64_t inner, uint64_t outer, uint32_t box_inner) {
    auto enc = encode_fn();
    if (!enc) GG_FAIL(GAPGPU_ERR_CUDA, "cuTensorMapEncodeTiled is not available from the driver");
    cuuint64_t dims[2] = {inner, outer};
    cuuint64_t strides[1] = {inner * (cuuint64_t)esize};
    cuuint32_t box[2] = {box_inner, 128};
    cuuint32_t es[2] = {1, 1};
    CUresult r = enc(tm, dt, 2, base, dims, strides, box, es, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                        CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                                        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) GG_FAIL(GAPGPU_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")");
    return GAPGPU_OK;
}

template <int MODE, int EPI>
int launch(gapgpu_context& c, const CUtensorMap& a0, const CUtensorMap& a1, const CUtensorMap& b0, const CUtensorMap& b1,
           int ntile_n, int rows, int kchunks, const EpiParams& ep, int* err) {
    using Cf = Cfg<MODE>;
    const int smem = Cf::STAGES * Cf::STAGE + 1024;
    GG_CUDA(cudaFuncSetAttribute(k_tc_gemm<MODE, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    dim3 grid(ntile_n, (rows + BM - 1) / BM);
    k_tc_gemm<MODE, EPI><<<grid, THREADS, smem, c.stream>>>(a0, a1, b0, b1, kchunks, ep, err);
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

template <int MODE>
int run_mixed(gapgpu_context& c, const Coordinate& co, int nc) {
    using Cf = Cfg<MODE>;
    const int Dp = co.Dpad, Mp = co.Mpad;
    const size_t nq = (size_t)nc * Dp, nw = (size_t)nc * Mp;
    int rc;
    const int ntiles = Mp / BN;
    const size_t es = MODE == MODE_BF16X3 ? 2 : 4;
    if ((rc = c.Kbuf.ensure(es * nq)) || (rc = c.qlo.ensure(es * nq)) || (rc = c.Wbuf.ensure(es * nw)) ||
        (rc = c.Wlo.ensure(es * nw)) || (rc = c.epart.ensure(sizeof(double) * (size_t)nc * ntiles)) ||
        (rc = c.Gbuf.ensure(sizeof(float) * nq)) || (rc = c.total.ensure(sizeof(int) * 4)))
        return rc;
    int* err = c.total.as<int>() + 3;
    GG_CUDA(cudaMemsetAsync(err, 0, sizeof(int), c.stream));
    const int TB = 256;
    const unsigned nb = (unsigned)((nq + TB - 1) / TB);
    CUtensorMap a0, a1, b0, b1;
    const CUtensorMapDataType dt = MODE == MODE_BF16X3 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    if (MODE == MODE_BF16X3) {
        k_split_q<<<nb, TB, 0, c.stream>>>(nq, c.qbuf.as<float>(), c.Kbuf.as<__nv_bfloat16>(), c.qlo.as<__nv_bfloat16>());
        if ((rc = make_map(&a0, c.Kbuf.p, dt, 2, Dp, nc, Cf::KB)) || (rc = make_map(&a1, c.qlo.p, dt, 2, Dp, nc, Cf::KB)) ||
            (rc = make_map(&b0, co.dXhi, dt, 2, Dp, Mp, Cf::KB)) || (rc = make_map(&b1, co.dXlo, dt, 2, Dp, Mp, Cf::KB)))
            return rc;
    } else {
        k_round_q<<<nb, TB, 0, c.stream>>>(nq, c.qbuf.as<float>(), c.qlo.as<float>());
        if ((rc = make_map(&a0, c.qlo.p, dt, 4, Dp, nc, Cf::KB)) || (rc = make_map(&b0, co.dXf32, dt, 4, Dp, Mp, Cf::KB)))
            return rc;
        a1 = a0; b1 = b0;
    }
    c.launches++;
    double z = co.zeta;
    EpiParams ep{nc, Mp, co.dcoef32, (float)z, (z == std::floor(z) && z >= 1 && z <= 64) ? (int)z : 0, c.Wbuf.p, c.Wlo.p,
                 c.epart.as<double>(), ntiles};
    if ((rc = launch<MODE, EPI_KERNEL>(c, a0, a1, b0, b1, ntiles, nc, Dp / Cf::KB, ep, err))) return rc;
    k_rowsum_scatter32<<<(nc + 127) / 128, 128, 0, c.stream>>>(nc, ntiles, c.epart.as<double>(), c.centres.as<int>(),
                                                              c.eatom.as<double>());
    c.launches++;
    // GEMM2: G = W X, B operand = X^T rows (k = sparse index contiguous)
    if (MODE == MODE_BF16X3) {
        if ((rc = make_map(&a0, c.Wbuf.p, dt, 2, Mp, nc, Cf::KB)) || (rc = make_map(&a1, c.Wlo.p, dt, 2, Mp, nc, Cf::KB)) ||
            (rc = make_map(&b0, co.dXThi, dt, 2, Mp, Dp, Cf::KB)) || (rc = make_map(&b1, co.dXTlo, dt, 2, Mp, Dp, Cf::KB)))
            return rc;
    } else {
        if ((rc = make_map(&a0, c.Wbuf.p, dt, 4, Mp, nc, Cf::KB)) || (rc = make_map(&b0, co.dXTf32, dt, 4, Mp, Dp, Cf::KB)))
            return rc;
        a1 = a0; b1 = b0;
    }
    EpiParams ep2{nc, Dp, nullptr, 0.f, 0, c.Gbuf.p, nullptr, nullptr, 0};
    if ((rc = launch<MODE, EPI_STORE>(c, a0, a1, b0, b1, Dp / BN, nc, Mp / Cf::KB, ep2, err))) return rc;
    int herr = 0;
    GG_CUDA(cudaMemcpyAsync(&herr, err, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    GG_CUDA(cudaStreamSynchronize(c.stream));
    if (herr) GG_FAIL(GAPGPU_ERR_TIMEOUT, "tensor-core GEMM: a bounded mbarrier wait expired (code " + std::to_string(herr) + ")");
    return GAPGPU_OK;
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
    }
    return GAPGPU_OK;
}

int gp_mixed(gapgpu_context& c, const Coordinate& co, int nc, int precision) {
    if (nc == 0) return GAPGPU_OK;
    if (co.cov != COV_DOT_PRODUCT) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "SOAP coordinates need the dot_product covariance");
    if (co.Dpad % BN || co.Mpad % BN) GG_FAIL(GAPGPU_ERR_ARG, "internal: operand padding is not a multiple of 128");
    return precision == GAPGPU_MIXED_BF16X3 ? run_mixed<MODE_BF16X3>(c, co, nc) : run_mixed<MODE_TF32>(c, co, nc);
}

}  // namespace gapgpu
