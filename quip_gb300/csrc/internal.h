// internal.h -- shared types of libgapgpu (host and device).
#pragma once
#include <cstdint>
#include <cstddef>
#include <string>
#include <vector>
#include <map>
#include <cuda_runtime.h>

#include "../../include/gapgpu.h"

namespace gapgpu {

constexpr int MAX_SPECIES = 8;
constexpr int MAX_CENTRE_Z = 16;
constexpr int MAX_NMAX = 16;
constexpr int MAX_LMAX = 12;

enum DescType { DESC_SOAP = 1, DESC_DISTANCE_2B = 2 };
enum CovType { COV_ARD_SE = 1, COV_DOT_PRODUCT = 2 };

// Error reporting: thread-local message, status codes of gapgpu.h.
void set_error(const std::string& msg);
#define GG_FAIL(code, msg)                 \
    do {                                   \
        ::gapgpu::set_error(msg);          \
        return code;                       \
    } while (0)
#define GG_CUDA(call)                                                                                   \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess)                                                                          \
            GG_FAIL(GAPGPU_ERR_CUDA, std::string("CUDA error ") + cudaGetErrorString(e_) + " at " + #call); \
    } while (0)

// SOAP hyper-parameters plus the FP64 radial transform (host copy).
struct SoapParams {
    double rc = 0, w = 0.5, sigma = 1.0, alpha = 2.0, cw = 1.0, sigma0 = 0.0, bee = 10.0;
    int l_max = 4, n_max = 4, n_species = 1, n_Z = 1;
    int species_Z[MAX_SPECIES] = {0};
    int Z[MAX_CENTRE_Z] = {0};
    bool normalise = true, diagonal_radial = false, central_all = false;
    std::vector<double> rb, T;       // grid (n_max) and transform T[a*n_max + n]
    std::vector<double> centre_R;    // central-atom l=0 radial coefficient per n (incl. Y00, weight)
    int n_pairs() const;             // number of (ia, jb) rows of the power spectrum
    int dim() const { return n_pairs() * (l_max + 1) + 1; }
};

// Flat constant block passed by value to the SOAP kernels.
struct SoapConst {
    double rc, w, alpha, sigma0;
    int l_max, n_max, n_species, n_pairs, dim, dpad, ncomp;  // ncomp = n_species*n_max*(l_max+1)^2
    int normalise;
    int species_Z[MAX_SPECIES];
    double rb[MAX_NMAX];
    double T[MAX_NMAX * MAX_NMAX];
    double centre_R[MAX_NMAX];
    int centre_all;
    // Per-warp task lists of the forward kernel's neighbour-function phase (lane =
    // neighbour), longest first to the least-loaded of the 8 warps.  Task id a < n_max:
    // radial row a; n_max + m: Ylm column m; 0xff ends a list.
    unsigned char fsched[8][8];
};

struct Coordinate {
    int type = 0;
    SoapParams soap;
    double d2_rc = 0, d2_w = 0.5;
    int d2_Z1 = 0, d2_Z2 = 0;
    int cov = 0;
    double delta = 1.0, zeta = 1.0, signal_mean = 0.0;
    std::vector<double> theta;
    int M = 0, D = 0, Dpad = 0, Mpad = 0;
    std::vector<double> X, alpha, sc;   // X[s*D + d]
    std::string desc_str;
    double cutoff() const { return type == DESC_SOAP ? soap.rc : d2_rc; }
    // device copies
    double* dX64 = nullptr;     // [Mpad][Dpad] FP64, zero padded
    double* dcoef = nullptr;    // [Mpad] alpha*sparseCutoff*delta^2 (0 in padding)
    float* dXf32 = nullptr;     // [Mpad][Dpad] FP32 (TF32 operand)
    uint16_t* dXhi = nullptr;   // [Mpad][Dpad] BF16 hi
    uint16_t* dXlo = nullptr;   // [Mpad][Dpad] BF16 lo
    float* dXTf32 = nullptr;    // [Dpad][Mpad] transposed operands for the second GEMM
    uint16_t* dXTh16 = nullptr;  // [Dpad][Mpad] FP16 (coef zeta / f16_scale) x: the FP16 second GEMM's operand
    uint16_t* dXh16 = nullptr;   // [Mpad][Dpad] FP16 x: the FP16 first GEMM's operand
    double f16_scale = 0.0;      // S of W' = S K^(zeta-1); 0: no FP16 second GEMM for this coordinate
    uint16_t* dXThi = nullptr;
    uint16_t* dXTlo = nullptr;
    float* dcoef32 = nullptr;
    double* dtheta = nullptr;   // distance_2b
    double* dVarL = nullptr;    // [M][M] Cholesky factor of K_MM + lambda I (column-major lower), variance only
    void* dtab[2] = {nullptr, nullptr};  // SOAP constant block (soap_tab layout): [0] FP64, [1] FP32
};

}  // namespace gapgpu

struct gapgpu_model {
    std::vector<gapgpu::Coordinate> coords;
    double e0[128] = {0};
    double E_scale = 1.0;
    double cutoff = 0.0;
    std::string label;
    int xml_version = 0;
    int device = 0;
    bool var_requested = false, var_ready = false;  // init arg gap_variance_regularisation given / set up
    double var_reg = 0.001;
    double* de0 = nullptr;  // e0 per Z on the device
};

namespace gapgpu {
// model.cpp
int parse_model(const char* xml, size_t len, const char* init_args, const char* base_dir, gapgpu_model& m);
int upload_model(gapgpu_model& m);
void free_model_device(gapgpu_model& m);
std::map<std::string, std::string> parse_args(const std::string& s);
void soap_setup(SoapParams& s);
SoapConst soap_const(const Coordinate& c);
// soap.cu
int upload_soap_tables(Coordinate& co);
}  // namespace gapgpu
