// gp64.cu -- K5 plain path: the sparse-GP kernel sum in FP64.
//
// gp_predict (GAP gp_predict_module, absent from the reference checkout; called per
// descriptor instance at src/Potentials/IPModel_GAP.f95:447) evaluates, for the
// dot_product covariance, e_i = sum_s alpha_s delta^2 sc_s (q_i . x_s)^zeta and
// gradPredict_i = sum_s alpha_s delta^2 sc_s zeta (q_i . x_s)^(zeta-1) x_s.
// The reference does one GEMV per atom; here all centres go through two GEMMs:
//   K = Q X^T            [nc x M]   (epilogue: W = coef zeta K^(zeta-1), per-tile e sums)
//   G = W X              [nc x D]   (= gradPredict for every centre)
// with coef_s = alpha_s * sparseCutoff_s * delta^2.  FP64 SIMT tiles: GB300 has no
// fast FP64 tensor path, so this kernel is bounded by the FP64 FMA rate.
#include <cmath>
#include "context.h"

namespace gapgpu {
namespace {

constexpr int BM = 64, BN = 64, BK = 16, TPB = 256;

__device__ __forceinline__ double ipow(double x, int n) {
    double r = 1.0;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

// C[m, n] = sum_k A[m, k] B[n, k]  (both operands k-contiguous), epilogue on C.
// EPI: W = coef zeta C^(zeta-1) stored to W; epart[m, tile] = sum_n coef C^zeta.
__global__ void __launch_bounds__(TPB) k_gemm_nt_epi(int Mrows, int Ncols, int K, const double* __restrict__ A, int lda,
                                                     const double* __restrict__ B, int ldb, const double* __restrict__ coef,
                                                     double zeta, int izeta, double* __restrict__ W, int ldw,
                                                     double* __restrict__ epart, int ntiles) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN + 1];
    __shared__ double red[16][BM];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int e = threadIdx.x; e < BM * BK; e += TPB) {
            int r = e / BK, kk = e % BK;
            int gm = m0 + r, gk = k0 + kk;
            As[kk][r] = (gm < Mrows && gk < K) ? A[(size_t)gm * lda + gk] : 0.0;
            int gn = n0 + r;
            Bs[kk][r] = (gn < Ncols && gk < K) ? B[(size_t)gn * ldb + gk] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
    // epilogue
    double rs[4] = {0, 0, 0, 0};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int gm = m0 + ty + 16 * i;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int gn = n0 + tx + 16 * j;
            if (gm < Mrows && gn < Ncols) {
                double kv = acc[i][j], cf = coef[gn];
                double km1 = izeta > 0 ? ipow(kv, izeta - 1) : pow(kv, zeta - 1.0);
                W[(size_t)gm * ldw + gn] = cf * zeta * km1;
                rs[i] += cf * km1 * kv;
            } else if (gm < Mrows && gn < ldw) {
                W[(size_t)gm * ldw + gn] = 0.0;
            }
        }
    }
    // deterministic row sums over the tile's 64 columns: fixed-order reduction over tx
#pragma unroll
    for (int i = 0; i < 4; ++i) red[tx][ty + 16 * i] = rs[i];
    __syncthreads();
    if (threadIdx.x < BM) {
        int r = threadIdx.x;
        double s = 0;
        for (int t = 0; t < 16; ++t) s += red[t][r];
        if (m0 + r < Mrows) epart[(size_t)(m0 + r) * ntiles + blockIdx.x] = s;
    }
}

// C[m, n] = sum_k A[m, k] B[k, n]  (A k-contiguous, B n-contiguous).
__global__ void __launch_bounds__(TPB) k_gemm_nn(int Mrows, int Ncols, int K, const double* __restrict__ A, int lda,
                                                 const double* __restrict__ B, int ldb, double* __restrict__ C, int ldc) {
    __shared__ double As[BK][BM + 1];
    __shared__ double Bs[BK][BN];
    const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
    const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += BK) {
        for (int e = threadIdx.x; e < BM * BK; e += TPB) {
            int r = e / BK, kk = e % BK;
            int gm = m0 + r, gk = k0 + kk;
            As[kk][r] = (gm < Mrows && gk < K) ? A[(size_t)gm * lda + gk] : 0.0;
            int kb = e / BN, cn = e % BN;
            int gk2 = k0 + kb, gn = n0 + cn;
            Bs[kb][cn] = (gk2 < K && gn < Ncols) ? B[(size_t)gk2 * ldb + gn] : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        int gm = m0 + ty + 16 * i;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            int gn = n0 + tx + 16 * j;
            if (gm < Mrows && gn < Ncols) C[(size_t)gm * ldc + gn] = acc[i][j];
        }
    }
}

// e_i = sum over tiles (fixed order); eatom[centre] += e_i (one writer per centre).
__global__ void k_rowsum_scatter(int nc, int ntiles, const double* __restrict__ epart, const int* __restrict__ centres,
                                 double* __restrict__ ecent, double* __restrict__ eatom) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nc) return;
    double s = 0;
    for (int t = 0; t < ntiles; ++t) s += epart[(size_t)i * ntiles + t];
    ecent[i] = s;
    eatom[centres[i]] += s;
}

}  // namespace

int gp_fp64(gapgpu_context& c, const Coordinate& co, int nc) {
    if (nc == 0) return GAPGPU_OK;
    if (co.cov != COV_DOT_PRODUCT) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "SOAP coordinates need the dot_product covariance");
    const int M = co.M, Mp = co.Mpad, Dp = co.Dpad;
    const int ntiles = (M + BN - 1) / BN;
    int rc;
    if ((rc = c.Wbuf.ensure(sizeof(double) * (size_t)nc * Mp)) || (rc = c.epart.ensure(sizeof(double) * (size_t)nc * ntiles)) ||
        (rc = c.ecent.ensure(sizeof(double) * nc)) || (rc = c.Gbuf.ensure(sizeof(double) * (size_t)nc * Dp)))
        return rc;
    double z = co.zeta;
    int iz = (z == std::floor(z) && z >= 1 && z <= 64) ? (int)z : 0;
    dim3 g1(ntiles, (nc + BM - 1) / BM);
    k_gemm_nt_epi<<<g1, TPB, 0, c.stream>>>(nc, M, co.soap.dim(), c.qbuf.as<double>(), Dp, co.dX64, Dp, co.dcoef, z, iz,
                                            c.Wbuf.as<double>(), Mp, c.epart.as<double>(), ntiles);
    k_rowsum_scatter<<<(nc + 127) / 128, 128, 0, c.stream>>>(nc, ntiles, c.epart.as<double>(), c.cur_centres,
                                                            c.ecent.as<double>(), c.eatom.as<double>());
    dim3 g2((Dp + BN - 1) / BN, (nc + BM - 1) / BM);
    k_gemm_nn<<<g2, TPB, 0, c.stream>>>(nc, Dp, M, c.Wbuf.as<double>(), Mp, co.dX64, Dp, c.Gbuf.as<double>(), Dp);
    c.launches += 3;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

}  // namespace gapgpu
