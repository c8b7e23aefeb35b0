// context.h -- per-stream evaluation context: device workspace kept between calls.
#pragma once
#include <vector>
#include <string>
#include "internal.h"

namespace gapgpu {

#ifdef __CUDACC__
// FP32 -> TF32 operand, round to nearest (ties away), low 13 mantissa bits zero
__device__ __forceinline__ float round_tf32(float x) {
    uint32_t r;
    asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
    return __uint_as_float(r);
}
#endif

// A growable device buffer.
struct DBuf {
    void* p = nullptr;
    size_t cap = 0;
    int ensure(size_t bytes);
    template <class T> T* as() const { return static_cast<T*>(p); }
    void release();
};

// Host-side geometry derived from the lattice (connection_calc_connect set-up).
struct CellGeom {
    double lat[9], g[9], lat_eff[9], lat_eff_inv[9], lat_off[3];
    int cellsN[3], img[3], pbc[3];
    int ncell;
};

// Geometry record of one structure for the neighbour kernels (connection_calc_connect
// set-up: effective lattice, cell grid, image ranges, FP32 pre-filter constants).
struct GeomDev {
    double lat[9], lat_eff_inv[9], lat_off[3], cutoff;
    double origin[3];     // Cartesian corner of the effective cell (non-periodic axes)
    double ginv[9];       // inverse of the true lattice
    float lat32[9];       // FP32 lattice (hi part)
    float lat_lo[9];      // lattice - lat32 (lo part), for the mixed path's displacements
    float lim2;           // (cutoff + margin)^2: FP32 distances above it are certainly outside
    float sure2;          // (cutoff - margin)^2: FP32 distances below it are certainly inside
    int cellsN[3], img[3], pbc[3];
    int cell_base;        // first global cell index of this structure
    int atom_begin, atom_end;
};

struct Timings { float neighbours = 0, soap_fwd = 0, gemm = 0, soap_bwd = 0, pair2b = 0, reduce = 0, total = 0; };

}  // namespace gapgpu

struct gapgpu_context {
    const gapgpu_model* model = nullptr;
    int precision = GAPGPU_FP64;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // atoms
    gapgpu::DBuf pos, Z, mask, out_e, out_f, out_le, out_lv;
    // cells and neighbours
    gapgpu::DBuf cell_key, cell_key2, atom_idx, atom_idx2, cell_start, cell_end, ms, cub_tmp, minmax;
    gapgpu::DBuf nbr_cnt, nbr_off, nbr_j, nbr_d, nbr_s, nbr_rev, nbr_i, wpos, total, geoms, sid, dispmax, phi, plo;
    bool nbr_mixed = false;  // displacements of the last build in FP32 error-free arithmetic (mixed path)
    std::vector<gapgpu::GeomDev> h_geoms;  // geometry of the structures of the last neighbour build
    int n_atoms_built = 0;
    // per pair / per atom accumulators
    gapgpu::DBuf fpair, epair, eatom, redpart;
    // SOAP / GP workspace
    gapgpu::DBuf flags, centres, ncent, qbuf, qlo, pnorm, Kbuf, Wbuf, Wlo, epart, ecent, Gbuf, scratch;
    gapgpu::DBuf hbuf, a2c;                   // FP32 SOAP backward: h per centre, atom -> centre
    int* cur_centres = nullptr;               // centre list of the coordinate being evaluated
    std::vector<int> nc_coord;                // centres per coordinate (prepare phase)
    gapgpu::DBuf chunks, schunk;              // segmented-reduction tables (per batch)
    // calc arguments of the current evaluation (IPModel_GAP.f95:334-335): only_descriptor
    // (given, 1-based value) and energy_per_coordinate
    bool sel_coord = false, want_epc = false, epc_valid = false;
    int only_coord = 0;
    gapgpu::DBuf epc_out, epca, epcp;         // [nstruct x ncoord]; per-atom and per-pair scratch
    // GAP variance of the last gapgpu_calc that requested it (local_gap_variance / print_gap_variance):
    // per-atom variances, minus their gradients, scratch, instance variances per coordinate
    bool want_var = false, var_valid = false, var_has_grad = false;
    gapgpu::DBuf var_le, var_f, var_lv, var_zero, var_info, var_q, var_k, var_y, var_g, var_inst;
    std::vector<long long> var_inst_off;
    void* blas = nullptr;                     // cuBLAS and cuSOLVER handles of the variance pass
    void* solver = nullptr;
    std::vector<int> h_chunks, h_schunk;
    int nstruct = 0, n_total = 0;
    // CUDA graph of the evaluation phase, keyed by shapes and buffer addresses
    cudaGraphExec_t graph = nullptr;
    std::vector<uintptr_t> graph_key, last_key;
    int graph_mode = 0;                       // 0: never, 1: capture on the second identical call
    bool autotune = true;                     // time the GEMM tile candidates of a new shape once
    int gemm_pairs = 1;                       // CTA-pair GEMM tiles: 0 off, 1 autotuner candidates, 2 only
    int soap_fwd_fixed = 1;                   // FP32 SOAP forward: 1 the fixed-size kernel where the basis has an instance
    int soap_bwd_nb = 1;                      // FP32 SOAP backward: 1 h kernel + one thread per pair where the basis allows, 0 one block per centre
    bool gemm2_f16 = false;                   // TF32 mode: FP16 second GEMM where the model allows it
    bool gemm1_f16 = false;                   // ... and FP16 first GEMM (on for GAPGPU_MIXED_F16 contexts)
    long long graph_hits = 0, graph_launches = 0;
    // stage timing (CUDA events): neighbour build, then the evaluation's stage boundaries
    bool timed = true, stage_valid = false, nbr_timed = false;
    cudaEvent_t nev[2] = {};
    cudaEvent_t cev[64] = {};
    int ncev = 0;
    // last results
    long long n_pairs = 0;
    long long launches = 0;
    gapgpu::Timings t;
    std::vector<gapgpu::DBuf*> buffers() {
        return {&pos, &Z, &mask, &out_e, &out_f, &out_le, &out_lv, &cell_key, &cell_key2, &atom_idx, &atom_idx2,
                &cell_start, &cell_end, &ms, &cub_tmp, &minmax, &nbr_cnt, &nbr_off, &nbr_j, &nbr_d, &nbr_s, &nbr_rev,
                &nbr_i, &wpos, &total, &geoms, &sid, &dispmax, &phi, &plo, &fpair, &epair, &eatom, &redpart, &flags, &centres,
                &ncent, &qbuf, &qlo, &pnorm, &Kbuf, &Wbuf, &Wlo, &epart, &ecent, &Gbuf, &scratch, &chunks, &schunk,
                &epc_out, &epca, &epcp, &hbuf, &a2c, &var_le, &var_f, &var_lv, &var_zero, &var_info, &var_q, &var_k, &var_y,
                &var_g, &var_inst};
    }
    std::vector<const gapgpu::DBuf*> buffers() const {
        std::vector<gapgpu::DBuf*> b = const_cast<gapgpu_context*>(this)->buffers();
        return std::vector<const gapgpu::DBuf*>(b.begin(), b.end());
    }
    ~gapgpu_context();
};

namespace gapgpu {
// neighbours.cu
int build_neighbours(gapgpu_context& c, int n, const double* d_pos, const double* lattice, const int* pbc, double cutoff,
                     const int* d_Z_for_check);
int build_neighbours_batch(gapgpu_context& c, int nstruct, const int* n_atoms, const double* d_pos, const double* lattices,
                           const int* pbcs, double cutoff, bool mixed = false);
int refresh_distances(gapgpu_context& c, const double* d_pos);
int load_external_neighbours(gapgpu_context& c, int n, const std::vector<int>& off, const std::vector<int>& nj,
                             const double* lattice, bool mixed);
int max_displacement(gapgpu_context& c, const double* d_pos, const double* d_ref, int n, double* out);
// calc.cu
enum ListMode { LIST_BUILD = 0, LIST_REFRESH = 1, LIST_GIVEN = 2 };
int prepare(gapgpu_context& c, int nstruct, const int* n_atoms, const double* lattices, const int* pbcs, const int* d_mask,
            double cutoff, int list_mode, int precision);
int run_evaluation(gapgpu_context& c, int precision, const int* d_mask);
int check_device_flags(gapgpu_context& c);
// soap.cu
int soap_forward(gapgpu_context& c, const Coordinate& co, int n, int nc);
int soap_backward(gapgpu_context& c, const Coordinate& co, int n, int nc);
int select_centres(gapgpu_context& c, const Coordinate& co, int n, const int* d_mask, int* nc_out);
// gp.cu
int gp_fp64(gapgpu_context& c, const Coordinate& co, int nc);
int gp_mixed(gapgpu_context& c, const Coordinate& co, int nc, int precision);
// pair.cu
int pair_2b(gapgpu_context& c, const std::vector<const Coordinate*>& coords, const int* d_mask);
// energy_per_coordinate: coordinate k's sum of e_i * covariance_cutoff per structure into
// epc_out[s * ncoord + k] -- SOAP from the per-centre energies in ecent, distance_2b from
// one pass over the pairs
int epc_soap(gapgpu_context& c, int k, int nc, int n);
int epc_pair(gapgpu_context& c, const Coordinate& co, int k, const int* d_mask);
bool coordinate_chosen(const gapgpu_context& c, int k);
// TF32 path with CTA pairs: the first GEMM K = Q X^T in FP16 (the forward kernel then writes
// the descriptors in FP16) when the model's FP16 operands exist
bool gemm1_f16_active(const gapgpu_context& c, const Coordinate& co);
int gather_outputs(gapgpu_context& c, const gapgpu_model& m, int n, const int* d_mask);
// the per-atom gather of fpair / epair / eatom into given outputs (no mask, e0 per Z given)
int gather_into(gapgpu_context& c, int n, const double* e0, double escale, double* le, double* F, double* LV);
// variance.cu: GAP variance estimate (set-up per model, pass after an evaluation)
int variance_setup(gapgpu_model& m, double reg);
int variance_eval(gapgpu_context& c, const int* d_mask, bool grad);
void destroy_handles(gapgpu_context& c);
}  // namespace gapgpu
