// calc.cu -- the C ABI (include/gapgpu.h) and the evaluation pipeline.
//
// Pipeline of one calculation (IPModel_GAP_Calc, src/Potentials/IPModel_GAP.f95:233-605,
// with the connection built first as potential_calc does, Potential.f95:844-858):
//   K1 neighbours -> per coordinate { SOAP: centres, K3/K4 forward, K5 GP GEMMs,
//   K4^T/K7 backward | distance_2b: K6 } -> K7/K8 gather + reductions.
// All device work is issued on the context's stream; host synchronisation happens only
// where a size must be known (pair count, centre count) and at the end of gapgpu_calc.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "context.h"

namespace gapgpu {
const char* last_error();

namespace {

size_t round_up(size_t v, size_t m) { return (v + m - 1) / m * m; }

__global__ void k_f64_to_f32(size_t n, const double* __restrict__ a, float* __restrict__ b) {
    size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (i < n) b[i] = (float)a[i];
}

struct ArgOpts {
    int precision = -1;
    bool bad_scale = false;
};

int parse_calc_args(const char* args, ArgOpts& o) {
    if (!args) return GAPGPU_OK;
    auto a = parse_args(args);
    if (a.count("r_scale") || a.count("E_scale")) {
        o.bad_scale = true;
        GG_FAIL(GAPGPU_ERR_ARG,
                "IPModel_GAP_Calc: rescaling of potential at the calc() stage with r_scale and E_scale not yet implemented!");
    }
    if (a.count("precision")) {
        const std::string& p = a["precision"];
        if (p == "fp64") o.precision = GAPGPU_FP64;
        else if (p == "bf16x3") o.precision = GAPGPU_MIXED_BF16X3;
        else if (p == "tf32") o.precision = GAPGPU_MIXED_TF32;
        else GG_FAIL(GAPGPU_ERR_ARG, "precision must be fp64, bf16x3 or tf32");
    }
    for (const char* k : {"local_gap_variance", "print_gap_variance", "energy_per_coordinate", "only_descriptor"}) {
        auto it = a.find(k);
        if (it != a.end() && it->second != "" && it->second != "F" && it->second != "0")
            GG_FAIL(GAPGPU_ERR_UNSUPPORTED, std::string("calc option ") + k + " is not supported by this library");
    }
    return GAPGPU_OK;
}

int check_device() {
    int ndev = 0;
    cudaError_t e = cudaGetDeviceCount(&ndev);
    if (e != cudaSuccess || ndev == 0) GG_FAIL(GAPGPU_ERR_CUDA, "no CUDA device available (this library has no CPU fallback)");
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp pr;
    GG_CUDA(cudaGetDeviceProperties(&pr, dev));
    if (pr.major < 10) GG_FAIL(GAPGPU_ERR_CUDA, "this library is built for sm_103a (GB300); found an older GPU");
    return GAPGPU_OK;
}

struct StageTimer {
    gapgpu_context& c;
    int k = 0;
    explicit StageTimer(gapgpu_context& c_) : c(c_) {
        if (!c.events) {
            for (auto& e : c.ev) cudaEventCreate(&e);
            c.events = true;
        }
    }
    void mark() {
        if (k < 8) cudaEventRecord(c.ev[k++], c.stream);
    }
};

}  // namespace

int upload_model(gapgpu_model& m) {
    int rc;
    if ((rc = check_device())) return rc;
    cudaGetDevice(&m.device);
    for (Coordinate& co : m.coords) {
        co.Dpad = (int)round_up(co.D, 128);
        co.Mpad = (int)round_up(co.M, 128);
        std::vector<double> X((size_t)co.Mpad * co.Dpad, 0.0), coef(co.Mpad, 0.0);
        for (int s = 0; s < co.M; ++s) {
            for (int d = 0; d < co.D; ++d) X[(size_t)s * co.Dpad + d] = co.X[(size_t)s * co.D + d];
            coef[s] = co.alpha[s] * co.sc[s] * co.delta * co.delta;
        }
        if (co.type == DESC_DISTANCE_2B) {  // compact 1-D layout
            for (int s = 0; s < co.M; ++s) X[s] = co.X[s];
        }
        GG_CUDA(cudaMalloc(&co.dX64, sizeof(double) * X.size()));
        GG_CUDA(cudaMemcpy(co.dX64, X.data(), sizeof(double) * X.size(), cudaMemcpyHostToDevice));
        GG_CUDA(cudaMalloc(&co.dcoef, sizeof(double) * coef.size()));
        GG_CUDA(cudaMemcpy(co.dcoef, coef.data(), sizeof(double) * coef.size(), cudaMemcpyHostToDevice));
        if (co.type == DESC_SOAP) {
            int rc2;
            if ((rc2 = upload_soap_tables(co))) return rc2;
        }
    }
    return GAPGPU_OK;
}

void free_model_device(gapgpu_model& m) {
    for (Coordinate& co : m.coords) {
        for (void* p : {(void*)co.dX64, (void*)co.dcoef, (void*)co.dXf32, (void*)co.dXhi, (void*)co.dXlo, (void*)co.dXTf32,
                        (void*)co.dXThi, (void*)co.dXTlo, (void*)co.dcoef32, (void*)co.dtheta, co.dtab[0], co.dtab[1]})
            if (p) cudaFree(p);
        co.dtab[0] = co.dtab[1] = nullptr;
        co.dX64 = nullptr; co.dcoef = nullptr; co.dXf32 = nullptr; co.dXhi = nullptr; co.dXlo = nullptr;
        co.dXTf32 = nullptr; co.dXThi = nullptr; co.dXTlo = nullptr; co.dcoef32 = nullptr; co.dtheta = nullptr;
    }
}

int prepare_mixed_operands(gapgpu_model& m);  // tcgen05.cu

// The whole pipeline on device-resident positions (c.pos, c.Z, optional mask).
static int run_pipeline(gapgpu_context& c, int n, const double* lattice, const int* pbc, const int* d_mask, int precision) {
    const gapgpu_model& m = *c.model;
    int rc;
    StageTimer tm(c);
    tm.mark();
    if ((rc = build_neighbours(c, n, c.pos.as<double>(), lattice, pbc, m.cutoff, nullptr))) return rc;
    tm.mark();
    const size_t P = std::max<long long>(c.n_pairs, 1);
    if ((rc = c.fpair.ensure(sizeof(double) * 3 * P)) || (rc = c.epair.ensure(sizeof(double) * P)) ||
        (rc = c.eatom.ensure(sizeof(double) * std::max(n, 1))))
        return rc;
    GG_CUDA(cudaMemsetAsync(c.fpair.p, 0, sizeof(double) * 3 * P, c.stream));
    GG_CUDA(cudaMemsetAsync(c.epair.p, 0, sizeof(double) * P, c.stream));
    GG_CUDA(cudaMemsetAsync(c.eatom.p, 0, sizeof(double) * std::max(n, 1), c.stream));
    const int saved = c.precision;
    c.precision = precision;
    float t_fwd = 0, t_gemm = 0, t_bwd = 0, t_2b = 0;
    cudaEvent_t e0, e1, e2, e3;
    cudaEventCreate(&e0); cudaEventCreate(&e1); cudaEventCreate(&e2); cudaEventCreate(&e3);
    for (const Coordinate& co : m.coords) {
        if (co.type == DESC_SOAP) {
            int nc = 0;
            if ((rc = select_centres(c, co, n, d_mask, &nc))) break;
            cudaEventRecord(e0, c.stream);
            if ((rc = soap_forward(c, co, n, nc))) break;
            cudaEventRecord(e1, c.stream);
            rc = precision == GAPGPU_FP64 ? gp_fp64(c, co, nc) : gp_mixed(c, co, nc, precision);
            if (rc) break;
            cudaEventRecord(e2, c.stream);
            if ((rc = soap_backward(c, co, n, nc))) break;
            cudaEventRecord(e3, c.stream);
            cudaEventSynchronize(e3);
            float a, b, d;
            cudaEventElapsedTime(&a, e0, e1); cudaEventElapsedTime(&b, e1, e2); cudaEventElapsedTime(&d, e2, e3);
            t_fwd += a; t_gemm += b; t_bwd += d;
        } else {
            cudaEventRecord(e0, c.stream);
            if ((rc = pair_2b(c, co, n, d_mask))) break;
            cudaEventRecord(e1, c.stream);
            cudaEventSynchronize(e1);
            float a;
            cudaEventElapsedTime(&a, e0, e1);
            t_2b += a;
        }
    }
    cudaEventDestroy(e0); cudaEventDestroy(e1); cudaEventDestroy(e2); cudaEventDestroy(e3);
    c.precision = saved;
    if (rc) return rc;
    tm.mark();
    if ((rc = gather_outputs(c, m, n, d_mask))) return rc;
    tm.mark();
    GG_CUDA(cudaGetLastError());
    cudaEventSynchronize(c.ev[3]);
    float a = 0, b = 0, d = 0;
    cudaEventElapsedTime(&a, c.ev[0], c.ev[1]);
    cudaEventElapsedTime(&b, c.ev[2], c.ev[3]);
    cudaEventElapsedTime(&d, c.ev[0], c.ev[3]);
    c.t.neighbours = a; c.t.reduce = b; c.t.total = d;
    c.t.soap_fwd = t_fwd; c.t.gemm = t_gemm; c.t.soap_bwd = t_bwd; c.t.pair2b = t_2b;
    return GAPGPU_OK;
}

}  // namespace gapgpu

using namespace gapgpu;

gapgpu_context::~gapgpu_context() {
    for (DBuf* b : {&pos, &Z, &mask, &out_e, &out_f, &out_v, &out_le, &out_lv, &cell_key, &cell_key2, &atom_idx, &atom_idx2,
                    &cell_start, &cell_end, &ms, &cub_tmp, &minmax, &nbr_cnt, &nbr_off, &nbr_j, &nbr_d, &nbr_s, &nbr_rev, &nbr_i, &wpos,
                    &total, &fpair, &epair, &eatom, &redpart, &flags, &centres, &ncent, &coef, &qbuf, &qlo, &pnorm, &Kbuf, &Wbuf,
                    &Wlo, &epart, &ecent, &Gbuf, &scratch})
        b->release();
    if (events)
        for (auto& e : ev) cudaEventDestroy(e);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

extern "C" {

const char* gapgpu_last_error(void) { return gapgpu::last_error(); }

int gapgpu_model_create(const char* xml, size_t xml_len, const char* init_args, const char* base_dir, gapgpu_model** out) {
    if (!out) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_model_create: out is NULL");
    *out = nullptr;
    gapgpu_model* m = new gapgpu_model();
    int rc = parse_model(xml, xml_len ? xml_len : (xml ? std::strlen(xml) : 0), init_args, base_dir, *m);
    if (!rc) rc = upload_model(*m);
    if (!rc) rc = prepare_mixed_operands(*m);
    if (rc) {
        free_model_device(*m);
        delete m;
        return rc;
    }
    *out = m;
    return GAPGPU_OK;
}

int gapgpu_model_cutoff(const gapgpu_model* m, double* cutoff) {
    if (!m || !cutoff) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_model_cutoff: NULL argument");
    *cutoff = m->cutoff;
    return GAPGPU_OK;
}

int gapgpu_model_info(const gapgpu_model* m, int* n_coordinates, int* dims, int* n_sparse, int capacity) {
    if (!m) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_model_info: NULL model");
    if (n_coordinates) *n_coordinates = (int)m->coords.size();
    for (int k = 0; k < (int)m->coords.size() && k < capacity; ++k) {
        if (dims) dims[k] = m->coords[k].D;
        if (n_sparse) n_sparse[k] = m->coords[k].M;
    }
    return GAPGPU_OK;
}

void gapgpu_model_destroy(gapgpu_model* m) {
    if (!m) return;
    free_model_device(*m);
    delete m;
}

int gapgpu_context_create(const gapgpu_model* m, int precision, gapgpu_context** out) {
    if (!m || !out) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_context_create: NULL argument");
    if (precision < GAPGPU_FP64 || precision > GAPGPU_MIXED_TF32) GG_FAIL(GAPGPU_ERR_ARG, "unknown precision");
    int rc;
    if ((rc = check_device())) return rc;
    gapgpu_context* c = new gapgpu_context();
    c->model = m;
    c->precision = precision;
    cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        GG_FAIL(GAPGPU_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
    }
    c->own_stream = true;
    *out = c;
    return GAPGPU_OK;
}

int gapgpu_context_set_stream(gapgpu_context* c, void* s) {
    if (!c) GG_FAIL(GAPGPU_ERR_ARG, "NULL context");
    if (c->own_stream && c->stream) cudaStreamDestroy(c->stream);
    c->stream = static_cast<cudaStream_t>(s);
    c->own_stream = false;
    return GAPGPU_OK;
}

void gapgpu_context_destroy(gapgpu_context* c) { delete c; }

int gapgpu_context_sync(gapgpu_context* c) {
    if (!c) GG_FAIL(GAPGPU_ERR_ARG, "NULL context");
    GG_CUDA(cudaStreamSynchronize(c->stream));
    return GAPGPU_OK;
}

int gapgpu_calc(gapgpu_context* c, int n, const double* pos, const int32_t* Z, const double* lattice, const int32_t* pbc,
                const int32_t* atom_mask, double* energy, double* local_e, double* force, double* virial,
                double* local_virial, const char* args) {
    if (!c || n < 0 || (n > 0 && (!pos || !Z)) || !lattice || !pbc) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc: bad argument");
    c->launches = 0;
    ArgOpts o;
    int rc;
    if ((rc = parse_calc_args(args, o))) return rc;
    const int prec = o.precision >= 0 ? o.precision : c->precision;
    if (n == 0) {
        if (energy) *energy = 0;
        if (virial) std::memset(virial, 0, 9 * sizeof(double));
        return GAPGPU_OK;
    }
    if ((rc = c->pos.ensure(sizeof(double) * 3 * n)) || (rc = c->Z.ensure(sizeof(int) * n)) ||
        (rc = c->mask.ensure(sizeof(int) * n)))
        return rc;
    GG_CUDA(cudaMemcpyAsync(c->pos.p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    GG_CUDA(cudaMemcpyAsync(c->Z.p, Z, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    const int* dmask = nullptr;
    if (atom_mask) {
        GG_CUDA(cudaMemcpyAsync(c->mask.p, atom_mask, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
        dmask = c->mask.as<int>();
    }
    if ((rc = run_pipeline(*c, n, lattice, pbc, dmask, prec))) return rc;
    double red[10];
    GG_CUDA(cudaMemcpyAsync(red, c->out_e.p, sizeof red, cudaMemcpyDeviceToHost, c->stream));
    if (force) GG_CUDA(cudaMemcpyAsync(force, c->out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    if (local_e) GG_CUDA(cudaMemcpyAsync(local_e, c->out_le.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (local_virial)
        GG_CUDA(cudaMemcpyAsync(local_virial, c->out_lv.p, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost, c->stream));
    GG_CUDA(cudaStreamSynchronize(c->stream));
    if (energy) *energy = red[0];
    if (virial) std::memcpy(virial, red + 1, 9 * sizeof(double));
    return GAPGPU_OK;
}

int gapgpu_calc_device(gapgpu_context* c, int n, const double* d_pos, const int32_t* d_Z, const double* lattice,
                       const int32_t* pbc, double* d_energy, double* d_force, double* d_virial) {
    if (!c || n <= 0 || !d_pos || !d_Z || !lattice || !pbc) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_device: bad argument");
    c->launches = 0;
    int rc;
    if ((rc = c->pos.ensure(sizeof(double) * 3 * n)) || (rc = c->Z.ensure(sizeof(int) * n))) return rc;
    GG_CUDA(cudaMemcpyAsync(c->pos.p, d_pos, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, c->stream));
    GG_CUDA(cudaMemcpyAsync(c->Z.p, d_Z, sizeof(int) * n, cudaMemcpyDeviceToDevice, c->stream));
    if ((rc = run_pipeline(*c, n, lattice, pbc, nullptr, c->precision))) return rc;
    if (d_energy) GG_CUDA(cudaMemcpyAsync(d_energy, c->out_e.p, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (d_virial)
        GG_CUDA(cudaMemcpyAsync(d_virial, c->out_e.as<double>() + 1, 9 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (d_force) GG_CUDA(cudaMemcpyAsync(d_force, c->out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, c->stream));
    return GAPGPU_OK;
}

int gapgpu_neighbours(gapgpu_context* c, int n, const double* pos, const double* lattice, const int32_t* pbc, double cutoff,
                      int32_t* offsets, int32_t* nbr_j, int32_t* nbr_shift, int64_t capacity, int64_t* total) {
    if (!c || n <= 0 || !pos || !lattice || !pbc) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_neighbours: bad argument");
    int rc;
    if ((rc = c->pos.ensure(sizeof(double) * 3 * n))) return rc;
    GG_CUDA(cudaMemcpyAsync(c->pos.p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    if ((rc = build_neighbours(*c, n, c->pos.as<double>(), lattice, pbc, cutoff, nullptr))) return rc;
    if (total) *total = c->n_pairs;
    if (offsets) GG_CUDA(cudaMemcpyAsync(offsets, c->nbr_off.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, c->stream));
    if (capacity >= c->n_pairs && c->n_pairs > 0) {
        if (nbr_j) GG_CUDA(cudaMemcpyAsync(nbr_j, c->nbr_j.p, sizeof(int) * c->n_pairs, cudaMemcpyDeviceToHost, c->stream));
        if (nbr_shift) {
            std::vector<int> packed(c->n_pairs);
            GG_CUDA(cudaMemcpyAsync(packed.data(), c->nbr_s.p, sizeof(int) * c->n_pairs, cudaMemcpyDeviceToHost, c->stream));
            GG_CUDA(cudaStreamSynchronize(c->stream));
            for (long long p = 0; p < c->n_pairs; ++p) {
                int s = packed[p];
                nbr_shift[3 * p] = (s & 1023) - 512;
                nbr_shift[3 * p + 1] = ((s >> 10) & 1023) - 512;
                nbr_shift[3 * p + 2] = ((s >> 20) & 1023) - 512;
            }
        }
    }
    GG_CUDA(cudaStreamSynchronize(c->stream));
    return GAPGPU_OK;
}

int gapgpu_descriptors(gapgpu_context* c, int coordinate, int n, const double* pos, const int32_t* Z, const double* lattice,
                       const int32_t* pbc, double* q, int64_t capacity, int* n_centres) {
    if (!c || n <= 0 || !pos || !Z || !lattice || !pbc) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_descriptors: bad argument");
    const gapgpu_model& m = *c->model;
    if (coordinate < 0 || coordinate >= (int)m.coords.size()) GG_FAIL(GAPGPU_ERR_ARG, "coordinate out of range");
    const Coordinate& co = m.coords[coordinate];
    if (co.type != DESC_SOAP) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "gapgpu_descriptors: coordinate is not SOAP");
    int rc;
    if ((rc = c->pos.ensure(sizeof(double) * 3 * n)) || (rc = c->Z.ensure(sizeof(int) * n))) return rc;
    GG_CUDA(cudaMemcpyAsync(c->pos.p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    GG_CUDA(cudaMemcpyAsync(c->Z.p, Z, sizeof(int) * n, cudaMemcpyHostToDevice, c->stream));
    if ((rc = build_neighbours(*c, n, c->pos.as<double>(), lattice, pbc, co.cutoff(), nullptr))) return rc;
    int nc = 0;
    if ((rc = select_centres(*c, co, n, nullptr, &nc))) return rc;
    if ((rc = soap_forward(*c, co, n, nc))) return rc;
    if (n_centres) *n_centres = nc;
    const int dim = co.soap.dim();
    if (q && capacity >= (int64_t)nc * dim && nc > 0) {
        if (c->precision == GAPGPU_FP64) {
            GG_CUDA(cudaMemcpy2DAsync(q, sizeof(double) * dim, c->qbuf.p, sizeof(double) * co.Dpad, sizeof(double) * dim, nc,
                                      cudaMemcpyDeviceToHost, c->stream));
        } else {
            std::vector<float> tmp((size_t)nc * dim);
            GG_CUDA(cudaMemcpy2DAsync(tmp.data(), sizeof(float) * dim, c->qbuf.p, sizeof(float) * co.Dpad, sizeof(float) * dim,
                                      nc, cudaMemcpyDeviceToHost, c->stream));
            GG_CUDA(cudaStreamSynchronize(c->stream));
            for (size_t k = 0; k < tmp.size(); ++k) q[k] = tmp[k];
        }
    }
    GG_CUDA(cudaStreamSynchronize(c->stream));
    return GAPGPU_OK;
}

int gapgpu_context_timings(const gapgpu_context* c, double* ms, int capacity) {
    if (!c || !ms) return 0;
    double v[7] = {c->t.neighbours, c->t.soap_fwd, c->t.gemm, c->t.soap_bwd, c->t.pair2b, c->t.reduce, c->t.total};
    int k = std::min(capacity, 7);
    for (int i = 0; i < k; ++i) ms[i] = v[i];
    return k;
}

int gapgpu_context_launches(const gapgpu_context* c, int64_t* launches) {
    if (!c || !launches) GG_FAIL(GAPGPU_ERR_ARG, "NULL argument");
    *launches = c->launches;
    return GAPGPU_OK;
}

}  // extern "C"
