// context.h -- per-stream evaluation context: device workspace kept between calls.
#pragma once
#include <vector>
#include <string>
#include "internal.h"

namespace gapgpu {

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

struct Timings { float neighbours = 0, soap_fwd = 0, gemm = 0, soap_bwd = 0, pair2b = 0, reduce = 0, total = 0; };

}  // namespace gapgpu

struct gapgpu_context {
    const gapgpu_model* model = nullptr;
    int precision = GAPGPU_FP64;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    // atoms
    gapgpu::DBuf pos, Z, mask, out_e, out_f, out_v, out_le, out_lv;
    // cells and neighbours
    gapgpu::DBuf cell_key, cell_key2, atom_idx, atom_idx2, cell_start, cell_end, ms, cub_tmp, minmax;
    gapgpu::DBuf nbr_cnt, nbr_off, nbr_j, nbr_d, nbr_s, nbr_rev, nbr_i, wpos, total;
    // per pair / per atom accumulators
    gapgpu::DBuf fpair, epair, eatom, redpart;
    // SOAP / GP workspace
    gapgpu::DBuf flags, centres, ncent, coef, qbuf, qlo, pnorm, Kbuf, Wbuf, Wlo, epart, ecent, Gbuf, scratch;
    // last results
    long long n_pairs = 0;
    long long launches = 0;
    gapgpu::Timings t;
    cudaEvent_t ev[8] = {};
    bool events = false;
    ~gapgpu_context();
};

namespace gapgpu {
// neighbours.cu
int build_neighbours(gapgpu_context& c, int n, const double* d_pos, const double* lattice, const int* pbc, double cutoff,
                     const int* d_Z_for_check);
// soap.cu
int soap_forward(gapgpu_context& c, const Coordinate& co, int n, int nc);
int soap_backward(gapgpu_context& c, const Coordinate& co, int n, int nc);
int select_centres(gapgpu_context& c, const Coordinate& co, int n, const int* d_mask, int* nc_out);
// gp.cu
int gp_fp64(gapgpu_context& c, const Coordinate& co, int nc);
int gp_mixed(gapgpu_context& c, const Coordinate& co, int nc, int precision);
// pair.cu
int pair_2b(gapgpu_context& c, const Coordinate& co, int n, const int* d_mask);
int gather_outputs(gapgpu_context& c, const gapgpu_model& m, int n, const int* d_mask);
}  // namespace gapgpu
