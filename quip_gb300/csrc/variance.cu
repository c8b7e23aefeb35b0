// variance.cu -- GAP variance estimate: the calc arguments local_gap_variance and
// print_gap_variance (src/Potentials/IPModel_GAP.f95:330-335, :464-488, :506-516) with the
// estimator set up from the init argument gap_variance_regularisation (:170-187).
//
// The estimator is GAP's gpCoordinates_initialise_variance_estimate / gp_predict variance
// (GAP gp_predict_module, absent from the reference checkout), restated from the published
// sparse-GP predictive variance:
//   C = K_MM + lambda I          (K_st = k(x_s, x_t), lambda = gap_variance_regularisation)
//   sigma^2(x) = k(x, x) - k^T C^-1 k,    k_s = k(x, x_s)   (no alpha, no sparseCutoff)
//   grad sigma^2 = grad k(x, x) - 2 (grad k)^T C^-1 k
// with k the coordinate's covariance: delta^2 (x.y)^zeta for SOAP, delta^2 exp(-(r - x_s)^2 /
// (2 theta^2)) for distance_2b.  It is accumulated as the reference does:
//   local_gap_variance(a)      += sigma^2 fc^2 / |ci|  for every instance with a in ci
//   gap_variance_gradient(:,j) += grad sigma^2 . dx/dr_j fc^2 + 2 sigma^2 fc dfc/dr_j
// Everything runs in FP64 (a variance is a difference of nearly equal numbers): C is
// formed with cuBLAS DGEMM and factorised with cuSOLVER's Cholesky once per model; per
// calculation each SOAP coordinate's descriptors are formed again, k by DGEMM, C^-1 k by the
// Cholesky solve, and sigma^2's gradient is chained back to the atoms by the SOAP backward
// kernel with dE/dq replaced by d sigma^2 / dq; the per-pair terms of distance_2b come from
// one kernel.  The deterministic gather of the energy path then assembles the per-atom
// variances and their gradients (no atomics).
#include <cublas_v2.h>
#include <cusolverDn.h>

#include <cmath>
#include <cstring>
#include <vector>

#include "context.h"

namespace gapgpu {
namespace {

constexpr int VAR_2B_MAX = 64;  // sparse points of a distance_2b coordinate the per-pair solve holds

#define GG_BLAS(call)                                                                     \
    do {                                                                                  \
        cublasStatus_t s_ = (call);                                                       \
        if (s_ != CUBLAS_STATUS_SUCCESS)                                                  \
            GG_FAIL(GAPGPU_ERR_CUDA, std::string("cuBLAS error ") + std::to_string((int)s_) + " at " + #call); \
    } while (0)
#define GG_SOLVER(call)                                                                   \
    do {                                                                                  \
        cusolverStatus_t s_ = (call);                                                     \
        if (s_ != CUSOLVER_STATUS_SUCCESS)                                                \
            GG_FAIL(GAPGPU_ERR_CUDA, std::string("cuSOLVER error ") + std::to_string((int)s_) + " at " + #call); \
    } while (0)

// x^z, by repeated multiplication for a small integer exponent iz > 0 (zeta of the models)
__device__ __forceinline__ double powz(double x, double z, int iz) {
    if (iz > 0) {
        double r = 1.0;
        for (int k = 0; k < iz; ++k) r *= x;
        return r;
    }
    if (z == 0.0) return 1.0;
    return pow(x, z);
}
int int_exponent(double z) { return (z == std::floor(z) && z >= 1 && z <= 64) ? (int)z : 0; }

// C = delta^2 K^zeta + reg I in place (K = X X^T, column-major M x M)
__global__ void k_cov_dot(int M, double* __restrict__ C, double d2, double zeta, int iz, double reg) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)M * M) return;
    double v = d2 * powz(C[k], zeta, iz);
    if (k % M == k / M) v += reg;
    C[k] = v;
}
// C_st = delta^2 exp(-(x_s - x_t)^2 / (2 theta^2)) + reg delta_st (distance_2b: one value per sparse point)
__global__ void k_cov_1d(int M, const double* __restrict__ X, double* __restrict__ C, double d2, double it2, double reg) {
    const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= (long long)M * M) return;
    const int s = (int)(k % M), t = (int)(k / M);
    const double u = X[s] - X[t];
    C[k] = d2 * exp(-0.5 * u * u * it2) + (s == t ? reg : 0.0);
}

__global__ void k_to_double(size_t n, const float* __restrict__ in, double* __restrict__ out) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = in[i];
}
__global__ void k_to_float(size_t n, const double* __restrict__ in, float* __restrict__ out) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) out[i] = (float)in[i];
}

// Y = delta^2 K^zeta (the right-hand sides of the solve), K column-major M x nc
__global__ void k_kvec(size_t n, const double* __restrict__ K, double* __restrict__ Y, double d2, double zeta, int iz) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) Y[i] = d2 * powz(K[i], zeta, iz);
}

// Per centre i (one block): sigma^2 = delta^2 (q.q)^zeta - sum_s delta^2 K_si^zeta Y_si, Y = C^-1 k;
// the centre's variance goes to eatom (fc = 1, ci = the centre) and to the instance list.
__global__ void k_sigma(int M, int D, int Dpad, const double* __restrict__ Q, const double* __restrict__ K,
                        const double* __restrict__ Y, double d2, double zeta, int iz, const int* __restrict__ centres,
                        double* __restrict__ eatom, double* __restrict__ inst) {
    __shared__ double s_a[256], s_b[256];
    const int i = blockIdx.x;
    double kk = 0, qq = 0;
    for (int s = threadIdx.x; s < M; s += blockDim.x) kk += d2 * powz(K[(size_t)i * M + s], zeta, iz) * Y[(size_t)i * M + s];
    for (int d = threadIdx.x; d < D; d += blockDim.x) qq += Q[(size_t)i * Dpad + d] * Q[(size_t)i * Dpad + d];
    s_a[threadIdx.x] = kk;
    s_b[threadIdx.x] = qq;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            s_a[threadIdx.x] += s_a[threadIdx.x + st];
            s_b[threadIdx.x] += s_b[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const double v = d2 * powz(s_b[0], zeta, iz) - s_a[0];
        inst[i] = v;
        eatom[centres[i]] += v;
    }
}

// W = -2 Y delta^2 zeta K^(zeta-1) in place over Y (the weights of grad sigma^2 = X^T W + ...)
__global__ void k_weights(size_t n, const double* __restrict__ K, double* __restrict__ Y, double d2, double zeta, int iz) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) Y[i] = -2.0 * Y[i] * d2 * zeta * powz(K[i], zeta - 1.0, iz > 0 ? iz - 1 : 0);
}

// G[i] += delta^2 zeta (q.q)^(zeta-1) 2 q_i (grad of k(x, x)); padding columns zeroed
__global__ void k_gdiag(int D, int Dpad, const double* __restrict__ Q, double* __restrict__ G, double d2, double zeta,
                        int iz) {
    __shared__ double s_q[256];
    __shared__ double s_f;
    const int i = blockIdx.x;
    double qq = 0;
    for (int d = threadIdx.x; d < D; d += blockDim.x) qq += Q[(size_t)i * Dpad + d] * Q[(size_t)i * Dpad + d];
    s_q[threadIdx.x] = qq;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) s_q[threadIdx.x] += s_q[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) s_f = d2 * zeta * powz(s_q[0], zeta - 1.0, iz > 0 ? iz - 1 : 0) * 2.0;
    __syncthreads();
    for (int d = threadIdx.x; d < Dpad; d += blockDim.x)
        G[(size_t)i * Dpad + d] = d < D ? G[(size_t)i * Dpad + d] + s_f * Q[(size_t)i * Dpad + d] : 0.0;
}

// distance_2b: one thread per directed pair p = (a -> b) of a centre a in the mask; for a
// coordinate that takes the pair, sigma^2 of r_ab by the Cholesky solve in registers,
// epair[p] += sigma^2 fc^2 / 2 (the instance's variance split over ci = (a, b)) and, with
// the gradient, fpair[p] += (d sigma^2/dr fc^2 + 2 sigma^2 fc dfc/dr) r_hat (its derivative
// with respect to r_b; minus that with respect to r_a).
struct Var2b {
    double rc, w, d2, it2;
    int Z1, Z2, M;
    const double* X;
    const double* L;  // Cholesky factor, column-major lower
    double* inst;     // [P]: sigma^2 of the pair as an instance of this coordinate, NaN otherwise
};
__device__ __forceinline__ void fcut64(double r, double rc, double w, double& f, double& df) {
    if (r > rc) { f = 0; df = 0; return; }
    if (r > rc - w) {
        const double pi = 3.14159265358979323846;
        const double a = pi * (r - rc + w) / w;
        f = 0.5 * (cos(a) + 1.0);
        df = -0.5 * pi * sin(a) / w;
        return;
    }
    f = 1; df = 0;
}
__global__ void k_var_2b(long long P, const int* __restrict__ Z, const int* __restrict__ mask, const int* __restrict__ ni,
                         const int* __restrict__ nj, const double4* __restrict__ nd, Var2b v, bool grad,
                         double* __restrict__ fpair, double* __restrict__ epair) {
    const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P) return;
    v.inst[p] = __longlong_as_double(0x7ff8000000000000LL);
    const int a = ni[p], b = nj[p];
    if (mask && !mask[a]) return;
    const double4 d = nd[p];
    if (d.w >= v.rc) return;
    const int za = Z[a], zb = Z[b];
    const bool zi1 = v.Z1 == 0 || za == v.Z1, zj2 = v.Z2 == 0 || zb == v.Z2;
    const bool zi2 = v.Z2 == 0 || za == v.Z2, zj1 = v.Z1 == 0 || zb == v.Z1;
    if (!((zi1 && zj2) || (zi2 && zj1))) return;
    const double r = d.w;
    const int M = v.M;
    double k[VAR_2B_MAX], y[VAR_2B_MAX];
    for (int s = 0; s < M; ++s) {
        const double u = r - v.X[s];
        k[s] = v.d2 * exp(-0.5 * u * u * v.it2);
    }
    for (int i = 0; i < M; ++i) {  // L z = k
        double t = k[i];
        for (int j = 0; j < i; ++j) t -= v.L[i + (size_t)j * M] * y[j];
        y[i] = t / v.L[i + (size_t)i * M];
    }
    for (int i = M - 1; i >= 0; --i) {  // L^T y = z
        double t = y[i];
        for (int j = i + 1; j < M; ++j) t -= v.L[j + (size_t)i * M] * y[j];
        y[i] = t / v.L[i + (size_t)i * M];
    }
    double var = v.d2, dvar = 0;
    for (int s = 0; s < M; ++s) {
        var -= k[s] * y[s];
        dvar += -2.0 * y[s] * k[s] * (v.X[s] - r) * v.it2;
    }
    double fc, dfc;
    fcut64(r, v.rc, v.w, fc, dfc);
    v.inst[p] = var;
    epair[p] += 0.5 * var * fc * fc;
    if (grad) {
        const double g = (dvar * fc * fc + 2.0 * var * fc * dfc) / r;
        fpair[3 * (size_t)p] += g * d.x;
        fpair[3 * (size_t)p + 1] += g * d.y;
        fpair[3 * (size_t)p + 2] += g * d.z;
    }
}

__global__ void k_negate(size_t n, double* __restrict__ x) {
    const size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) x[i] = -x[i];
}

unsigned nblk(size_t n, int tb) { return (unsigned)((n + tb - 1) / tb); }

int context_handles(gapgpu_context& c) {
    if (!c.blas) {
        cublasHandle_t h = nullptr;
        GG_BLAS(cublasCreate(&h));
        c.blas = h;
    }
    if (!c.solver) {
        cusolverDnHandle_t h = nullptr;
        GG_SOLVER(cusolverDnCreate(&h));
        c.solver = h;
    }
    GG_BLAS(cublasSetStream(static_cast<cublasHandle_t>(c.blas), c.stream));
    GG_SOLVER(cusolverDnSetStream(static_cast<cusolverDnHandle_t>(c.solver), c.stream));
    return GAPGPU_OK;
}

}  // namespace

void destroy_handles(gapgpu_context& c) {
    if (c.blas) cublasDestroy(static_cast<cublasHandle_t>(c.blas));
    if (c.solver) cusolverDnDestroy(static_cast<cusolverDnHandle_t>(c.solver));
    c.blas = c.solver = nullptr;
}

// C = K_MM + reg I and its Cholesky factor for every coordinate (init argument
// gap_variance_regularisation, IPModel_GAP.f95:185-187).
int variance_setup(gapgpu_model& m, double reg) {
    cublasHandle_t hb = nullptr;
    cusolverDnHandle_t hs = nullptr;
    double* work = nullptr;
    int* info = nullptr;
    int rc = GAPGPU_OK;
    auto done = [&](int code) {
        if (hb) cublasDestroy(hb);
        if (hs) cusolverDnDestroy(hs);
        if (work) cudaFree(work);
        if (info) cudaFree(info);
        return code;
    };
    if (cublasCreate(&hb) != CUBLAS_STATUS_SUCCESS || cusolverDnCreate(&hs) != CUSOLVER_STATUS_SUCCESS) {
        set_error("variance set-up: cuBLAS / cuSOLVER handles could not be created");
        return done(GAPGPU_ERR_CUDA);
    }
    if (cudaMalloc(&info, sizeof(int)) != cudaSuccess) {
        set_error("variance set-up: out of device memory");
        return done(GAPGPU_ERR_CUDA);
    }
    for (Coordinate& co : m.coords) {
        const int M = co.M;
        if (M < 1) continue;
        if (co.type == DESC_DISTANCE_2B && M > VAR_2B_MAX) {
            set_error("gap_variance_regularisation: a distance_2b coordinate has more than " + std::to_string(VAR_2B_MAX) +
                      " sparse points");
            return done(GAPGPU_ERR_UNSUPPORTED);
        }
        if (co.type == DESC_SOAP && co.cov != COV_DOT_PRODUCT) {
            set_error("gap_variance_regularisation: SOAP coordinates need the dot_product covariance");
            return done(GAPGPU_ERR_UNSUPPORTED);
        }
        if (cudaMalloc(&co.dVarL, sizeof(double) * (size_t)M * M) != cudaSuccess) {
            set_error("variance set-up: out of device memory for K_MM");
            return done(GAPGPU_ERR_CUDA);
        }
        const double d2 = co.delta * co.delta;
        if (co.type == DESC_SOAP) {
            const double one = 1.0, zero = 0.0;
            if (cublasDgemm(hb, CUBLAS_OP_T, CUBLAS_OP_N, M, M, co.D, &one, co.dX64, co.Dpad, co.dX64, co.Dpad, &zero,
                            co.dVarL, M) != CUBLAS_STATUS_SUCCESS) {
                set_error("variance set-up: cuBLAS DGEMM failed");
                return done(GAPGPU_ERR_CUDA);
            }
            k_cov_dot<<<nblk((size_t)M * M, 256), 256>>>(M, co.dVarL, d2, co.zeta, int_exponent(co.zeta), reg);
        } else {
            k_cov_1d<<<nblk((size_t)M * M, 256), 256>>>(M, co.dX64, co.dVarL, d2, 1.0 / (co.theta[0] * co.theta[0]), reg);
        }
        int lwork = 0;
        if (cusolverDnDpotrf_bufferSize(hs, CUBLAS_FILL_MODE_LOWER, M, co.dVarL, M, &lwork) != CUSOLVER_STATUS_SUCCESS) {
            set_error("variance set-up: cuSOLVER workspace query failed");
            return done(GAPGPU_ERR_CUDA);
        }
        if (work) cudaFree(work);
        work = nullptr;
        if (cudaMalloc(&work, sizeof(double) * (size_t)std::max(lwork, 1)) != cudaSuccess) {
            set_error("variance set-up: out of device memory");
            return done(GAPGPU_ERR_CUDA);
        }
        if (cusolverDnDpotrf(hs, CUBLAS_FILL_MODE_LOWER, M, co.dVarL, M, work, lwork, info) != CUSOLVER_STATUS_SUCCESS) {
            set_error("variance set-up: cuSOLVER Cholesky failed");
            return done(GAPGPU_ERR_CUDA);
        }
        int h_info = 0;
        cudaError_t e = cudaMemcpy(&h_info, info, sizeof(int), cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) {
            set_error(std::string("variance set-up: ") + cudaGetErrorString(e));
            return done(GAPGPU_ERR_CUDA);
        }
        if (h_info != 0) {
            set_error("gap_variance_regularisation: K_MM + regularisation I is not positive definite");
            return done(GAPGPU_ERR_ARG);
        }
    }
    m.var_ready = true;
    return done(rc);
}

// The variance pass after an evaluation (its outputs already assembled): per-atom
// variances into var_le and, with `grad`, minus their gradients into var_f.
int variance_eval(gapgpu_context& c, const int* d_mask, bool grad) {
    const gapgpu_model& m = *c.model;
    const int n = c.n_total, ncoord = (int)m.coords.size();
    int rc;
    if ((rc = context_handles(c))) return rc;
    cublasHandle_t hb = static_cast<cublasHandle_t>(c.blas);
    cusolverDnHandle_t hs = static_cast<cusolverDnHandle_t>(c.solver);
    const size_t P = std::max<long long>(c.n_pairs, 1);
    if ((rc = c.var_le.ensure(sizeof(double) * std::max(n, 1))) || (rc = c.var_f.ensure(sizeof(double) * 3 * std::max(n, 1))) ||
        (rc = c.var_lv.ensure(sizeof(double) * 9 * std::max(n, 1))) || (rc = c.var_zero.ensure(sizeof(double) * 128)) ||
        (rc = c.var_info.ensure(sizeof(int) * 4)))
        return rc;
    GG_CUDA(cudaMemsetAsync(c.var_zero.p, 0, sizeof(double) * 128, c.stream));
    GG_CUDA(cudaMemsetAsync(c.fpair.p, 0, sizeof(double) * 3 * P, c.stream));
    GG_CUDA(cudaMemsetAsync(c.epair.p, 0, sizeof(double) * P, c.stream));
    GG_CUDA(cudaMemsetAsync(c.eatom.p, 0, sizeof(double) * std::max(n, 1), c.stream));
    // instance variances: SOAP centres, then distance_2b pairs, per coordinate
    c.var_inst_off.assign(ncoord + 1, 0);
    size_t ninst = 0;
    for (int k = 0; k < ncoord; ++k) {
        c.var_inst_off[k] = (long long)ninst;
        if (coordinate_chosen(c, k)) ninst += m.coords[k].type == DESC_SOAP ? (size_t)c.nc_coord[k] : P;
    }
    c.var_inst_off[ncoord] = (long long)ninst;
    if ((rc = c.var_inst.ensure(sizeof(double) * std::max<size_t>(ninst, 1)))) return rc;
    const int saved = c.precision;
    for (int k = 0; k < ncoord && !rc; ++k) {
        const Coordinate& co = m.coords[k];
        if (!coordinate_chosen(c, k)) continue;
        const double d2 = co.delta * co.delta;
        double* inst = c.var_inst.as<double>() + c.var_inst_off[k];
        if (co.type == DESC_SOAP) {
            const int nc = c.nc_coord[k], M = co.M, D = co.D, Dp = co.Dpad;
            if (nc == 0 || M == 0) continue;
            c.cur_centres = c.centres.as<int>() + (size_t)k * n;
            if ((rc = soap_forward(c, co, n, nc))) break;
            const bool fp64 = c.precision == GAPGPU_FP64;
            const double* Q = c.qbuf.as<double>();
            if (!fp64) {
                if ((rc = c.var_q.ensure(sizeof(double) * (size_t)nc * Dp))) break;
                k_to_double<<<nblk((size_t)nc * Dp, 256), 256, 0, c.stream>>>((size_t)nc * Dp, c.qbuf.as<float>(),
                                                                            c.var_q.as<double>());
                Q = c.var_q.as<double>();
            }
            if ((rc = c.var_k.ensure(sizeof(double) * (size_t)M * nc)) || (rc = c.var_y.ensure(sizeof(double) * (size_t)M * nc)))
                break;
            const double one = 1.0, zero = 0.0;
            const int iz = int_exponent(co.zeta);
            // K (M x nc, column-major) = X Q^T: column i holds q_i . x_s
            GG_BLAS(cublasDgemm(hb, CUBLAS_OP_T, CUBLAS_OP_N, M, nc, D, &one, co.dX64, Dp, Q, Dp, &zero, c.var_k.as<double>(), M));
            const size_t nk = (size_t)M * nc;
            k_kvec<<<nblk(nk, 256), 256, 0, c.stream>>>(nk, c.var_k.as<double>(), c.var_y.as<double>(), d2, co.zeta, iz);
            GG_SOLVER(cusolverDnDpotrs(hs, CUBLAS_FILL_MODE_LOWER, M, nc, co.dVarL, M, c.var_y.as<double>(), M,
                                       c.var_info.as<int>()));
            k_sigma<<<nc, 256, 0, c.stream>>>(M, D, Dp, Q, c.var_k.as<double>(), c.var_y.as<double>(), d2, co.zeta, iz,
                                              c.cur_centres, c.eatom.as<double>(), inst);
            if (grad) {
                if ((rc = c.var_g.ensure(sizeof(double) * (size_t)nc * Dp))) break;
                k_weights<<<nblk(nk, 256), 256, 0, c.stream>>>(nk, c.var_k.as<double>(), c.var_y.as<double>(), d2, co.zeta, iz);
                // G (Dpad x nc) = X^T W: column i is sum_s W_si x_s
                GG_BLAS(cublasDgemm(hb, CUBLAS_OP_N, CUBLAS_OP_N, D, nc, M, &one, co.dX64, Dp, c.var_y.as<double>(), M, &zero,
                                    c.var_g.as<double>(), Dp));
                k_gdiag<<<nc, 256, 0, c.stream>>>(D, Dp, Q, c.var_g.as<double>(), d2, co.zeta, iz);
                // the SOAP backward with dE/dq replaced by d sigma^2 / dq, in the context's precision
                if ((rc = c.Gbuf.ensure((fp64 ? sizeof(double) : sizeof(float)) * (size_t)nc * Dp))) break;
                if (fp64)
                    GG_CUDA(cudaMemcpyAsync(c.Gbuf.p, c.var_g.p, sizeof(double) * (size_t)nc * Dp, cudaMemcpyDeviceToDevice,
                                            c.stream));
                else
                    k_to_float<<<nblk((size_t)nc * Dp, 256), 256, 0, c.stream>>>((size_t)nc * Dp, c.var_g.as<double>(),
                                                                                c.Gbuf.as<float>());
                if ((rc = soap_backward(c, co, n, nc))) break;
            }
        } else {
            const long long Pp = c.n_pairs;
            if (Pp == 0) continue;
            Var2b v{co.d2_rc, co.d2_w, d2, 1.0 / (co.theta[0] * co.theta[0]), co.d2_Z1, co.d2_Z2, co.M, co.dX64, co.dVarL,
                    inst};
            k_var_2b<<<nblk((size_t)Pp, 128), 128, 0, c.stream>>>(Pp, c.Z.as<int>(), d_mask, c.nbr_i.as<int>(),
                                                                  c.nbr_j.as<int>(), c.nbr_d.as<double4>(), v, grad,
                                                                  c.fpair.as<double>(), c.epair.as<double>());
        }
        GG_CUDA(cudaGetLastError());
    }
    c.precision = saved;
    if (rc) return rc;
    if ((rc = gather_into(c, n, c.var_zero.as<double>(), 1.0, c.var_le.as<double>(), c.var_f.as<double>(),
                          c.var_lv.as<double>())))
        return rc;
    // the gather gives minus the derivative of the summed variances (as forces are of E)
    k_negate<<<nblk(3 * (size_t)n, 256), 256, 0, c.stream>>>(3 * (size_t)n, c.var_f.as<double>());
    GG_CUDA(cudaGetLastError());
    c.var_valid = true;
    c.var_has_grad = grad;
    return GAPGPU_OK;
}

}  // namespace gapgpu

using namespace gapgpu;

extern "C" {

int gapgpu_gap_variance(gapgpu_context* c, double* local_variance, double* variance_gradient, int n) {
    if (!c) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance: NULL context");
    if (!c->var_valid)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance: the last calculation did not request local_gap_variance");
    if (n != c->n_total) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance: n differs from the last calculation's atoms");
    if (variance_gradient && !c->var_has_grad)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance: the last calculation computed no forces, so no variance gradient");
    if (local_variance)
        GG_CUDA(cudaMemcpyAsync(local_variance, c->var_le.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (variance_gradient)
        GG_CUDA(cudaMemcpyAsync(variance_gradient, c->var_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    GG_CUDA(cudaStreamSynchronize(c->stream));
    return GAPGPU_OK;
}

int gapgpu_gap_variance_instances(gapgpu_context* c, int coordinate, double* variance, double* fc2, int32_t* atom_i,
                                  int32_t* atom_j, int capacity, int* count) {
    if (!c || !count) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance_instances: NULL argument");
    if (!c->var_valid)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance_instances: the last calculation did not request the variance");
    const gapgpu_model& m = *c->model;
    if (coordinate < 0 || coordinate >= (int)m.coords.size())
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_gap_variance_instances: coordinate out of range");
    const long long o0 = c->var_inst_off[coordinate], o1 = c->var_inst_off[coordinate + 1];
    std::vector<double> v((size_t)(o1 - o0));
    if (!v.empty())
        GG_CUDA(cudaMemcpyAsync(v.data(), c->var_inst.as<double>() + o0, sizeof(double) * v.size(), cudaMemcpyDeviceToHost,
                                c->stream));
    const Coordinate& co = m.coords[coordinate];
    std::vector<int> ai, aj;
    std::vector<double4> dd;
    const int n = c->n_total;
    if (co.type == DESC_SOAP) {
        ai.resize(v.size());
        if (!v.empty())
            GG_CUDA(cudaMemcpyAsync(ai.data(), c->centres.as<int>() + (size_t)coordinate * n, sizeof(int) * v.size(),
                                    cudaMemcpyDeviceToHost, c->stream));
    } else if (!v.empty()) {
        ai.resize(v.size());
        aj.resize(v.size());
        dd.resize(v.size());
        GG_CUDA(cudaMemcpyAsync(ai.data(), c->nbr_i.p, sizeof(int) * v.size(), cudaMemcpyDeviceToHost, c->stream));
        GG_CUDA(cudaMemcpyAsync(aj.data(), c->nbr_j.p, sizeof(int) * v.size(), cudaMemcpyDeviceToHost, c->stream));
        GG_CUDA(cudaMemcpyAsync(dd.data(), c->nbr_d.p, sizeof(double4) * v.size(), cudaMemcpyDeviceToHost, c->stream));
    }
    GG_CUDA(cudaStreamSynchronize(c->stream));
    int k = 0;
    for (size_t q = 0; q < v.size(); ++q) {
        if (std::isnan(v[q])) continue;  // a pair that is not an instance of this coordinate
        if (k < capacity) {
            if (variance) variance[k] = v[q];
            double f = 1.0;
            if (co.type != DESC_SOAP) {
                const double r = dd[q].w, w = co.d2_w, rc = co.d2_rc;
                f = r > rc ? 0.0 : r > rc - w ? 0.5 * (std::cos(M_PI * (r - rc + w) / w) + 1.0) : 1.0;
            }
            if (fc2) fc2[k] = f * f;
            if (atom_i) atom_i[k] = ai[q];
            if (atom_j) atom_j[k] = co.type == DESC_SOAP ? -1 : aj[q];
        }
        ++k;
    }
    *count = k;
    return GAPGPU_OK;
}

}  // extern "C"
