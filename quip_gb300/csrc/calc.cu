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

struct ArgOpts {
    int precision = -1;
    bool bad_scale = false;
    bool select = false, epc = false;  // only_descriptor given; energy_per_coordinate requested
    bool var = false;                   // local_gap_variance / print_gap_variance requested
    int only = 0;
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
        else if (p == "fp16") o.precision = GAPGPU_MIXED_F16;
        else GG_FAIL(GAPGPU_ERR_ARG, "precision must be fp64, bf16x3, tf32 or fp16");
    }
    // local_gap_variance=<name> (a non-empty name) and print_gap_variance=T request the
    // variance estimate (IPModel_GAP.f95:330-335, :362-364)
    {
        auto lv = a.find("local_gap_variance");
        auto pv = a.find("print_gap_variance");
        const bool print = pv != a.end() && (pv->second == "" || pv->second == "T" || pv->second == "t" ||
                                              pv->second == "true" || pv->second == "True" || pv->second == "1");
        o.var = (lv != a.end() && !lv->second.empty()) || print;
    }
    // only_descriptor (IPModel_GAP.f95:334, :399-403): given at all, it selects the coordinate
    // of that 1-based index when the model has more than one
    auto od = a.find("only_descriptor");
    if (od != a.end()) {
        char* end = nullptr;
        const long v = std::strtol(od->second.c_str(), &end, 10);
        if (od->second.empty() || *end) GG_FAIL(GAPGPU_ERR_ARG, "only_descriptor must be an integer");
        o.select = true;
        o.only = (int)v;
    }
    // energy_per_coordinate=name (:335, :462, :570): a non-empty name requests the sums
    auto ep = a.find("energy_per_coordinate");
    o.epc = ep != a.end() && !ep->second.empty();
    return GAPGPU_OK;
}

// The precision a call's args give (precision=...), for that call only.  FP16 is the TF32
// mode with both FP16 GEMM options on, TF32 the same mode with them off; the context's own
// options come back when the call returns.
struct CallPrecision {
    gapgpu_context& c;
    bool g1, g2;
    int prec;
    CallPrecision(gapgpu_context& ctx, int requested) : c(ctx), g1(ctx.gemm1_f16), g2(ctx.gemm2_f16) {
        prec = requested < 0 ? c.precision : requested;
        if (requested == GAPGPU_MIXED_F16) {
            prec = GAPGPU_MIXED_TF32;
            c.gemm1_f16 = c.gemm2_f16 = true;
        } else if (requested == GAPGPU_MIXED_TF32) {
            c.gemm1_f16 = c.gemm2_f16 = false;
        }
    }
    ~CallPrecision() {
        c.gemm1_f16 = g1;
        c.gemm2_f16 = g2;
    }
};

void apply_call_opts(gapgpu_context& c, const ArgOpts& o) {
    c.sel_coord = o.select;
    c.only_coord = o.only;
    c.want_epc = o.epc;
    c.epc_valid = false;
    c.want_var = o.var;
    c.var_valid = false;
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

}  // namespace

// only_descriptor selects coordinate k (0-based) only when the model has more than one
// (IPModel_GAP.f95:399-403)
bool coordinate_chosen(const gapgpu_context& c, int k) {
    return !c.sel_coord || c.model->coords.size() <= 1 || k + 1 == c.only_coord;
}

bool gemm1_f16_active(const gapgpu_context& c, const Coordinate& co) {
    return c.precision == GAPGPU_MIXED_TF32 && c.gemm1_f16 && c.gemm_pairs >= 1 && co.dXh16 != nullptr;
}

int upload_model(gapgpu_model& m) {
    int rc;
    if ((rc = check_device())) return rc;
    cudaGetDevice(&m.device);
    GG_CUDA(cudaMalloc(&m.de0, sizeof(double) * 128));
    GG_CUDA(cudaMemcpy(m.de0, m.e0, sizeof(double) * 128, cudaMemcpyHostToDevice));
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
    if (m.de0) cudaFree(m.de0);
    m.de0 = nullptr;
    for (Coordinate& co : m.coords) {
        for (void* p : {(void*)co.dX64, (void*)co.dcoef, (void*)co.dXf32, (void*)co.dXhi, (void*)co.dXlo, (void*)co.dXTf32,
                        (void*)co.dXThi, (void*)co.dXTlo, (void*)co.dXTh16, (void*)co.dXh16, (void*)co.dcoef32,
                        (void*)co.dtheta, (void*)co.dVarL, co.dtab[0], co.dtab[1]})
            if (p) cudaFree(p);
        co.dVarL = nullptr;
        co.dtab[0] = co.dtab[1] = nullptr;
        co.dXTh16 = nullptr;
        co.dXh16 = nullptr;
        co.dX64 = nullptr; co.dcoef = nullptr; co.dXf32 = nullptr; co.dXhi = nullptr; co.dXlo = nullptr;
        co.dXTf32 = nullptr; co.dXThi = nullptr; co.dXTlo = nullptr; co.dcoef32 = nullptr; co.dtheta = nullptr;
    }
}

int prepare_mixed_operands(gapgpu_model& m);  // tcgen05.cu

namespace {
constexpr int RED_CHUNK = 512;  // atoms per first-level reduction block (relative to each structure's first atom)
}

// ---------------------------------------------------------------- phase A
// Neighbour list (rebuilt at `cutoff`, only its displacements refreshed when the list
// is kept, or already loaded from the caller), per-coordinate centre lists,
// segmented-reduction tables and the output buffers.  All host synchronisation of an
// evaluation happens here.
int prepare(gapgpu_context& c, int nstruct, const int* n_atoms, const double* lattices, const int* pbcs, const int* d_mask,
            double cutoff, int list_mode, int precision) {
    const bool rebuild = list_mode != LIST_REFRESH;
    const gapgpu_model& m = *c.model;
    int rc, n = 0;
    for (int s = 0; s < nstruct; ++s) n += n_atoms[s];
    const double* d_pos = c.pos.as<double>();
    c.nbr_timed = c.timed;
    if (c.timed) {
        for (cudaEvent_t& e : c.nev)
            if (!e) cudaEventCreate(&e);
        cudaEventRecord(c.nev[0], c.stream);
    }
    if (list_mode == LIST_BUILD) {
        if ((rc = build_neighbours_batch(c, nstruct, n_atoms, d_pos, lattices, pbcs, cutoff, precision != GAPGPU_FP64)))
            return rc;
    } else if (list_mode == LIST_REFRESH) {
        if (n != c.n_total || nstruct != c.nstruct) GG_FAIL(GAPGPU_ERR_ARG, "kept neighbour list does not match the atoms");
        if ((rc = refresh_distances(c, d_pos))) return rc;
    }
    if (c.timed) cudaEventRecord(c.nev[1], c.stream);
    if (!rebuild) return GAPGPU_OK;  // centres, tables and buffers are those of the build
    c.nstruct = nstruct;
    c.n_total = n;
    const int ncoord = (int)m.coords.size();
    if ((rc = c.centres.ensure(sizeof(int) * std::max<size_t>(1, (size_t)n * ncoord)))) return rc;
    c.nc_coord.assign(ncoord, 0);
    for (int k = 0; k < ncoord; ++k) {
        const Coordinate& co = m.coords[k];
        if (co.type != DESC_SOAP || n == 0) continue;
        c.cur_centres = c.centres.as<int>() + (size_t)k * n;
        if ((rc = select_centres(c, co, n, d_mask, &c.nc_coord[k]))) return rc;
    }
    // reduction tables: chunks of RED_CHUNK atoms counted from each structure's first atom
    c.h_chunks.clear();
    c.h_schunk.assign(nstruct + 1, 0);
    for (int s = 0, a0 = 0; s < nstruct; a0 += n_atoms[s], ++s) {
        c.h_schunk[s] = (int)c.h_chunks.size() / 2;
        for (int a = a0; a < a0 + n_atoms[s]; a += RED_CHUNK) {
            c.h_chunks.push_back(a);
            c.h_chunks.push_back(std::min(a0 + n_atoms[s], a + RED_CHUNK));
        }
    }
    c.h_schunk[nstruct] = (int)c.h_chunks.size() / 2;
    const size_t nch = std::max<size_t>(1, c.h_chunks.size() / 2);
    const size_t P = std::max<long long>(c.n_pairs, 1);
    if ((rc = c.chunks.ensure(sizeof(int2) * nch)) || (rc = c.schunk.ensure(sizeof(int) * (nstruct + 1))) ||
        (rc = c.redpart.ensure(sizeof(double) * 10 * nch)) || (rc = c.fpair.ensure(sizeof(double) * 3 * P)) ||
        (rc = c.epair.ensure(sizeof(double) * P)) || (rc = c.eatom.ensure(sizeof(double) * std::max(n, 1))) ||
        (rc = c.out_le.ensure(sizeof(double) * std::max(n, 1))) || (rc = c.out_f.ensure(sizeof(double) * 3 * std::max(n, 1))) ||
        (rc = c.out_lv.ensure(sizeof(double) * 9 * std::max(n, 1))) || (rc = c.out_e.ensure(sizeof(double) * 10 * nstruct)) ||
        (rc = c.total.ensure(sizeof(int) * 4)))
        return rc;
    if (!c.h_chunks.empty())
        GG_CUDA(cudaMemcpyAsync(c.chunks.p, c.h_chunks.data(), sizeof(int) * c.h_chunks.size(), cudaMemcpyHostToDevice,
                                c.stream));
    GG_CUDA(cudaMemcpyAsync(c.schunk.p, c.h_schunk.data(), sizeof(int) * (nstruct + 1), cudaMemcpyHostToDevice, c.stream));
    // the host vectors above must outlive the copies
    GG_CUDA(cudaStreamSynchronize(c.stream));
    return GAPGPU_OK;
}

namespace {

void record(gapgpu_context& c, bool timed) {
    if (!timed || c.ncev >= 64) return;
    if (!c.cev[c.ncev]) cudaEventCreate(&c.cev[c.ncev]);
    cudaEventRecord(c.cev[c.ncev++], c.stream);
}

// ---------------------------------------------------------------- phase B
// Stream work only (kernels, memsets): the part of an evaluation that a CUDA graph can
// capture.  With `timed`, events bracket the stages: [start] then per coordinate
// (fwd, gemm, bwd | pair) and [gather, end].
int evaluate(gapgpu_context& c, int precision, const int* d_mask, bool timed) {
    const gapgpu_model& m = *c.model;
    const int n = c.n_total;
    int rc = GAPGPU_OK;
    c.ncev = 0;
    record(c, timed);
    GG_CUDA(cudaMemsetAsync(c.total.as<int>() + 3, 0, sizeof(int), c.stream));
    if (n > 0) {
        const size_t P = std::max<long long>(c.n_pairs, 1);
        GG_CUDA(cudaMemsetAsync(c.fpair.p, 0, sizeof(double) * 3 * P, c.stream));
        GG_CUDA(cudaMemsetAsync(c.epair.p, 0, sizeof(double) * P, c.stream));
        GG_CUDA(cudaMemsetAsync(c.eatom.p, 0, sizeof(double) * n, c.stream));
        const int saved = c.precision;
        c.precision = precision;
        const int ncoord = (int)m.coords.size();
        if (c.want_epc) {
            if ((rc = c.epc_out.ensure(sizeof(double) * (size_t)ncoord * c.nstruct))) return rc;
            GG_CUDA(cudaMemsetAsync(c.epc_out.p, 0, sizeof(double) * (size_t)ncoord * c.nstruct, c.stream));
        }
        // the distance_2b coordinates run together, in one pass over the pairs, at the
        // position of the first of them
        std::vector<const Coordinate*> two_body;
        std::vector<int> two_body_k;
        for (int k = 0; k < ncoord; ++k)
            if (m.coords[k].type != DESC_SOAP && coordinate_chosen(c, k)) {
                two_body.push_back(&m.coords[k]);
                two_body_k.push_back(k);
            }
        bool two_body_done = false;
        for (int k = 0; k < ncoord && !rc; ++k) {
            const Coordinate& co = m.coords[k];
            if (!coordinate_chosen(c, k)) continue;
            if (co.type == DESC_SOAP) {
                const int nc = c.nc_coord[k];
                c.cur_centres = c.centres.as<int>() + (size_t)k * n;
                record(c, timed);
                if ((rc = soap_forward(c, co, n, nc))) break;
                record(c, timed);
                rc = precision == GAPGPU_FP64 ? gp_fp64(c, co, nc) : gp_mixed(c, co, nc, precision);
                if (!rc && c.want_epc) rc = epc_soap(c, k, nc, n);
                if (rc) break;
                record(c, timed);
                if ((rc = soap_backward(c, co, n, nc))) break;
            } else if (!two_body_done) {
                two_body_done = true;
                record(c, timed);
                if ((rc = pair_2b(c, two_body, d_mask))) break;
                for (size_t j = 0; j < two_body.size() && c.want_epc && !rc; ++j)
                    rc = epc_pair(c, *two_body[j], two_body_k[j], d_mask);
            }
        }
        c.precision = saved;
        if (rc) return rc;
        record(c, timed);
        if ((rc = gather_outputs(c, m, n, d_mask))) return rc;
    } else {
        GG_CUDA(cudaMemsetAsync(c.out_e.p, 0, sizeof(double) * 10 * c.nstruct, c.stream));
    }
    record(c, timed);
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

std::vector<uintptr_t> graph_key(const gapgpu_context& c, int precision, const int* d_mask) {
    std::vector<uintptr_t> k = {(uintptr_t)precision, (uintptr_t)d_mask, (uintptr_t)c.n_total, (uintptr_t)c.nstruct,
                                (uintptr_t)c.n_pairs, (uintptr_t)c.model, (uintptr_t)c.stream,
                                (uintptr_t)c.h_chunks.size(), (uintptr_t)c.sel_coord, (uintptr_t)(intptr_t)c.only_coord,
                                (uintptr_t)c.want_epc, (uintptr_t)c.gemm1_f16, (uintptr_t)c.gemm2_f16,
                                (uintptr_t)c.gemm_pairs};
    for (int nc : c.nc_coord) k.push_back((uintptr_t)nc);
    for (const gapgpu::DBuf* b : c.buffers()) k.push_back((uintptr_t)b->p);
    return k;
}

}  // namespace

// Phase B, replayed from a CUDA graph when the context's graph mode is on and the same
// shapes and buffers were seen on the previous call (capture on the second identical
// call, replay from the third).
int run_evaluation(gapgpu_context& c, int precision, const int* d_mask) {
    c.stage_valid = false;
    if (!c.graph_mode) {
        int rc = evaluate(c, precision, d_mask, c.timed);
        c.stage_valid = c.timed;
        return rc;
    }
    std::vector<uintptr_t> key = graph_key(c, precision, d_mask);
    if (c.graph && key == c.graph_key) {
        GG_CUDA(cudaGraphLaunch(c.graph, c.stream));
        c.launches += c.graph_launches;
        c.graph_hits++;
        return GAPGPU_OK;
    }
    if (key == c.last_key) {
        if (c.graph) {
            cudaGraphExecDestroy(c.graph);
            c.graph = nullptr;
        }
        const long long l0 = c.launches;
        GG_CUDA(cudaStreamBeginCapture(c.stream, cudaStreamCaptureModeRelaxed));
        int rc = evaluate(c, precision, d_mask, false);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(c.stream, &g);
        if (rc) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) GG_FAIL(GAPGPU_ERR_CUDA, std::string("CUDA graph capture: ") + cudaGetErrorString(e));
        e = cudaGraphInstantiate(&c.graph, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            c.graph = nullptr;
            GG_FAIL(GAPGPU_ERR_CUDA, std::string("CUDA graph instantiate: ") + cudaGetErrorString(e));
        }
        c.graph_key = key;
        c.graph_launches = c.launches - l0;
        GG_CUDA(cudaGraphLaunch(c.graph, c.stream));
        return GAPGPU_OK;
    }
    c.last_key = key;
    int rc = evaluate(c, precision, d_mask, c.timed);
    c.stage_valid = c.timed;
    return rc;
}

// Error bits left on the device by the last evaluation (overlapping atoms found by a
// distance refresh, an expired tensor-core wait); call after the stream is idle.
int check_device_flags(gapgpu_context& c) {
    int f[4] = {0, 0, 0, 0};
    GG_CUDA(cudaMemcpy(f, c.total.p, sizeof f, cudaMemcpyDeviceToHost));
    if (f[2] & 2) GG_FAIL(GAPGPU_ERR_ATOMS, "connection_calc_dists: atoms overlap exactly (distance below 1e-10)");
    if (f[3]) GG_FAIL(GAPGPU_ERR_TIMEOUT, "a bounded device-side mbarrier wait expired (code " + std::to_string(f[3]) + ")");
    return GAPGPU_OK;
}

}  // namespace gapgpu

namespace gapgpu {
namespace {

// FMA-rate probe: FMA_CHAINS independent chains per thread (enough to hide the FMA latency
// at 16 warps per SM), either as scalar fma.rn.f32 or as packed fma.rn.f32x2 on pairs.
// The sum is written only when it equals a value it cannot reach, so the loop stays.
constexpr int FMA_CHAINS = 8;
template <bool PACKED>
__global__ void __launch_bounds__(512) k_fma_rate(int iters, float seed, float* out) {
    float a[FMA_CHAINS];
#pragma unroll
    for (int j = 0; j < FMA_CHAINS; ++j) a[j] = seed + 1e-7f * (float)(threadIdx.x + j);
    const float m = 0.9999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
        if constexpr (PACKED) {
#pragma unroll
            for (int j = 0; j < FMA_CHAINS; j += 2) {
                unsigned long long x, mm, cc;
                asm("mov.b64 %0, {%1, %2};" : "=l"(x) : "f"(a[j]), "f"(a[j + 1]));
                asm("mov.b64 %0, {%1, %1};" : "=l"(mm) : "f"(m));
                asm("mov.b64 %0, {%1, %1};" : "=l"(cc) : "f"(c));
                asm("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x) : "l"(mm), "l"(cc));
                asm("mov.b64 {%0, %1}, %2;" : "=f"(a[j]), "=f"(a[j + 1]) : "l"(x));
            }
        } else {
#pragma unroll
            for (int j = 0; j < FMA_CHAINS; ++j) a[j] = fmaf(a[j], m, c);
        }
    }
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < FMA_CHAINS; ++j) s += a[j];
    if (s == -1.0f) out[blockIdx.x] = s;
}

}  // namespace
}  // namespace gapgpu

using namespace gapgpu;

gapgpu_context::~gapgpu_context() {
    for (DBuf* b : buffers()) b->release();
    for (cudaEvent_t e : nev)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : cev)
        if (e) cudaEventDestroy(e);
    if (graph) cudaGraphExecDestroy(graph);
    destroy_handles(*this);
    if (own_stream && stream) cudaStreamDestroy(stream);
}

namespace {

// Stage times of the last timed evaluation, from its events (waits for them).
void compute_timings(gapgpu_context& c) {
    Timings t;
    if (c.stage_valid && c.ncev >= 2) {
        cudaEventSynchronize(c.cev[c.ncev - 1]);
        auto el = [&](cudaEvent_t a, cudaEvent_t b) {
            float ms = 0;
            cudaEventElapsedTime(&ms, a, b);
            return ms;
        };
        int i = 1;
        bool two_body_done = false;
        t.reduce += el(c.cev[0], c.cev[1]);  // output zeroing
        for (int kc = 0; kc < (int)c.model->coords.size(); ++kc) {
            const Coordinate& co = c.model->coords[kc];
            if (!coordinate_chosen(c, kc)) continue;
            if (co.type == DESC_SOAP) {
                if (i + 3 >= c.ncev) break;
                t.soap_fwd += el(c.cev[i], c.cev[i + 1]);
                t.gemm += el(c.cev[i + 1], c.cev[i + 2]);
                t.soap_bwd += el(c.cev[i + 2], c.cev[i + 3]);
                i += 3;
            } else if (!two_body_done) {
                two_body_done = true;
                if (i + 1 >= c.ncev) break;
                t.pair2b += el(c.cev[i], c.cev[i + 1]);
                i += 1;
            }
        }
        if (i + 1 < c.ncev) t.reduce += el(c.cev[i], c.cev[i + 1]);
        t.total = el(c.cev[0], c.cev[c.ncev - 1]);
        if (c.nbr_timed) {
            t.neighbours = el(c.nev[0], c.nev[1]);
            t.total = el(c.nev[0], c.cev[c.ncev - 1]);
        }
    }
    c.t = t;
}

int copy_inputs(gapgpu_context& c, int n, const double* pos, const int32_t* Z, const int32_t* mask, cudaMemcpyKind kind) {
    int rc;
    if ((rc = c.pos.ensure(sizeof(double) * 3 * std::max(n, 1))) || (rc = c.Z.ensure(sizeof(int) * std::max(n, 1))) ||
        (rc = c.mask.ensure(sizeof(int) * std::max(n, 1))))
        return rc;
    if (n == 0) return GAPGPU_OK;
    GG_CUDA(cudaMemcpyAsync(c.pos.p, pos, sizeof(double) * 3 * n, kind, c.stream));
    GG_CUDA(cudaMemcpyAsync(c.Z.p, Z, sizeof(int) * n, kind, c.stream));
    if (mask) GG_CUDA(cudaMemcpyAsync(c.mask.p, mask, sizeof(int) * n, kind, c.stream));
    return GAPGPU_OK;
}

}  // namespace

extern "C" {

const char* gapgpu_last_error(void) { return gapgpu::last_error(); }

int gapgpu_model_create(const char* xml, size_t xml_len, const char* init_args, const char* base_dir, gapgpu_model** out) {
    if (!out) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_model_create: out is NULL");
    *out = nullptr;
    gapgpu_model* m = new gapgpu_model();
    int rc = parse_model(xml, xml_len ? xml_len : (xml ? std::strlen(xml) : 0), init_args, base_dir, *m);
    if (!rc) rc = upload_model(*m);
    if (!rc) rc = prepare_mixed_operands(*m);
    if (!rc && m->var_requested) rc = variance_setup(*m, m->var_reg);
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

int gapgpu_model_footprint(const gapgpu_model* m, int precision, int64_t n_atoms, double mean_neighbours, int64_t* bytes) {
    if (!m || !bytes || n_atoms < 0 || !(mean_neighbours >= 0)) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_model_footprint: bad argument");
    const double rs = precision == GAPGPU_FP64 ? 8.0 : 4.0;
    // per atom: positions, species, outputs, cell binning; per pair: list (j, d, shift,
    // reverse, i) and force/energy accumulators
    double per_atom = 3 * 8 + 4 + 8 * (1 + 3 + 9 + 1) + 7 * 4 + 16 + mean_neighbours * (4 + 32 + 4 + 4 + 4 + 24 + 8);
    double per_centre = 0;
    for (const Coordinate& co : m->coords) {
        if (co.type != DESC_SOAP) continue;
        const SoapParams& sp = co.soap;
        const double ncomp = (double)sp.n_species * sp.n_max * (sp.l_max + 1) * (sp.l_max + 1);
        const double Dp = ((co.D + 127) / 128) * 128.0, Mp = ((co.M + 127) / 128) * 128.0;
        double c = rs * (ncomp + 2 * Dp) + 8 + 4;          // c, q, G, norm, centre index
        if (precision == GAPGPU_FP64) c += 8 * Mp + 8 * (Mp / 64 + 1) + 8;
        else c += 2 * 4 * Dp + 2 * 4 * Mp + 8 * (Mp / 128);  // GEMM operands (hi/lo or TF32), W, tile sums
        per_centre = std::max(per_centre, c);              // coordinates run one after the other
    }
    *bytes = (int64_t)((per_atom + per_centre) * (double)n_atoms) + (64 << 20);
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
    if (precision < GAPGPU_FP64 || precision > GAPGPU_MIXED_F16) GG_FAIL(GAPGPU_ERR_ARG, "unknown precision");
    int rc;
    if ((rc = check_device())) return rc;
    gapgpu_context* c = new gapgpu_context();
    c->model = m;
    // FP16 GEMMs run inside the TF32 mode (same kernels, FP16 operands where the model allows)
    c->precision = precision == GAPGPU_MIXED_F16 ? GAPGPU_MIXED_TF32 : precision;
    c->gemm1_f16 = c->gemm2_f16 = precision == GAPGPU_MIXED_F16;
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

int gapgpu_energy_per_coordinate(gapgpu_context* c, double* out, int capacity, int* count) {
    if (!c || !out || !count) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_energy_per_coordinate: NULL argument");
    if (!c->epc_valid)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_energy_per_coordinate: the last evaluation did not request energy_per_coordinate");
    const int n = c->nstruct * (int)c->model->coords.size();
    *count = n;
    if (capacity < n) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_energy_per_coordinate: output too small");
    GG_CUDA(cudaMemcpyAsync(out, c->epc_out.p, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    GG_CUDA(cudaStreamSynchronize(c->stream));
    return GAPGPU_OK;
}

int gapgpu_context_set_option(gapgpu_context* c, const char* key, int value) {
    if (!c || !key) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_context_set_option: NULL argument");
    const std::string k(key);
    if (k == "graphs") c->graph_mode = value ? 1 : 0;
    else if (k == "timing") c->timed = value != 0;
    else if (k == "autotune") c->autotune = value != 0;
    else if (k == "gemm2_f16") c->gemm2_f16 = value != 0;
    else if (k == "gemm1_f16") c->gemm1_f16 = value != 0;
    else if (k == "soap_bwd") c->soap_bwd_nb = value != 0;
    else if (k == "soap_fwd") c->soap_fwd_fixed = value != 0;
    else if (k == "pairs") {
        if (value < 0 || value > 2) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_context_set_option: pairs must be 0, 1 or 2");
        c->gemm_pairs = value;
    }
    else if (k == "priority") {
        // the context's own stream, recreated at the device's highest (value != 0) or
        // default scheduling priority: kernels of higher-priority streams get free SMs first
        if (!c->own_stream) GG_FAIL(GAPGPU_ERR_ARG, "priority applies to the context's own stream only");
        int lo = 0, hi = 0;
        GG_CUDA(cudaDeviceGetStreamPriorityRange(&lo, &hi));
        GG_CUDA(cudaStreamSynchronize(c->stream));
        cudaStream_t s = nullptr;
        GG_CUDA(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, value ? hi : lo));
        cudaStreamDestroy(c->stream);
        c->stream = s;
    }
    else GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_context_set_option: unknown option " + k);
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
    apply_call_opts(*c, o);
    const CallPrecision cp(*c, o.precision);
    const int prec = cp.prec;
    if (n == 0) {
        if (energy) *energy = 0;
        if (virial) std::memset(virial, 0, 9 * sizeof(double));
        return GAPGPU_OK;
    }
    if (o.var && !c->model->var_ready)
        GG_FAIL(GAPGPU_ERR_ARG,
                "local_gap_variance / print_gap_variance need the init argument gap_variance_regularisation");
    if ((rc = copy_inputs(*c, n, pos, Z, atom_mask, cudaMemcpyHostToDevice))) return rc;
    const int* dmask = atom_mask ? c->mask.as<int>() : nullptr;
    if ((rc = prepare(*c, 1, &n, lattice, pbc, dmask, c->model->cutoff, LIST_BUILD, prec))) return rc;
    if ((rc = run_evaluation(*c, prec, dmask))) return rc;
    c->epc_valid = c->want_epc;
    if (o.var) {
        const int saved = c->precision;
        c->precision = prec;
        rc = variance_eval(*c, dmask, force || virial || local_virial);
        c->precision = saved;
        if (rc) return rc;
    }
    double red[10];
    GG_CUDA(cudaMemcpyAsync(red, c->out_e.p, sizeof red, cudaMemcpyDeviceToHost, c->stream));
    if (force) GG_CUDA(cudaMemcpyAsync(force, c->out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    if (local_e) GG_CUDA(cudaMemcpyAsync(local_e, c->out_le.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (local_virial)
        GG_CUDA(cudaMemcpyAsync(local_virial, c->out_lv.p, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost, c->stream));
    GG_CUDA(cudaStreamSynchronize(c->stream));
    if ((rc = check_device_flags(*c))) return rc;
    if (energy) *energy = red[0];
    if (virial) std::memcpy(virial, red + 1, 9 * sizeof(double));
    return GAPGPU_OK;
}

int gapgpu_calc_device(gapgpu_context* c, int n, const double* d_pos, const int32_t* d_Z, const double* lattice,
                       const int32_t* pbc, double* d_energy, double* d_force, double* d_virial) {
    if (!c || n <= 0 || !d_pos || !d_Z || !lattice || !pbc) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_device: bad argument");
    c->launches = 0;
    int rc;
    if ((rc = copy_inputs(*c, n, d_pos, d_Z, nullptr, cudaMemcpyDeviceToDevice))) return rc;
    if ((rc = prepare(*c, 1, &n, lattice, pbc, nullptr, c->model->cutoff, LIST_BUILD, c->precision))) return rc;
    apply_call_opts(*c, ArgOpts{});
    if ((rc = run_evaluation(*c, c->precision, nullptr))) return rc;
    if (d_energy) GG_CUDA(cudaMemcpyAsync(d_energy, c->out_e.p, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (d_virial)
        GG_CUDA(cudaMemcpyAsync(d_virial, c->out_e.as<double>() + 1, 9 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    if (d_force) GG_CUDA(cudaMemcpyAsync(d_force, c->out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, c->stream));
    return GAPGPU_OK;
}

int gapgpu_calc_batch(gapgpu_context* c, int nstruct, const int32_t* n_atoms, const double* pos, const int32_t* Z,
                      const double* lattices, const int32_t* pbcs, double* energies, double* forces, double* virials,
                      const char* args) {
    if (!c || nstruct < 1 || !n_atoms || !lattices || !pbcs) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_batch: bad argument");
    c->launches = 0;
    ArgOpts o;
    int rc;
    if ((rc = parse_calc_args(args, o))) return rc;
    if (o.var) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "the GAP variance is computed by gapgpu_calc (one structure per call)");
    apply_call_opts(*c, o);
    const CallPrecision cp(*c, o.precision);
    const int prec = cp.prec;
    long long n = 0;
    for (int s = 0; s < nstruct; ++s) {
        if (n_atoms[s] < 0) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_batch: negative atom count");
        n += n_atoms[s];
    }
    if (n > (1LL << 30)) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_batch: too many atoms");
    if (n > 0 && (!pos || !Z)) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_batch: NULL positions or species");
    if ((rc = copy_inputs(*c, (int)n, pos, Z, nullptr, cudaMemcpyHostToDevice))) return rc;
    if ((rc = prepare(*c, nstruct, n_atoms, lattices, pbcs, nullptr, c->model->cutoff, LIST_BUILD, prec))) return rc;
    if ((rc = run_evaluation(*c, prec, nullptr))) return rc;
    c->epc_valid = c->want_epc;
    std::vector<double> red(10 * (size_t)nstruct);
    GG_CUDA(cudaMemcpyAsync(red.data(), c->out_e.p, sizeof(double) * red.size(), cudaMemcpyDeviceToHost, c->stream));
    if (forces && n > 0)
        GG_CUDA(cudaMemcpyAsync(forces, c->out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    GG_CUDA(cudaStreamSynchronize(c->stream));
    if ((rc = check_device_flags(*c))) return rc;
    for (int s = 0; s < nstruct; ++s) {
        if (energies) energies[s] = red[10 * (size_t)s];
        if (virials) std::memcpy(virials + 9 * (size_t)s, &red[10 * (size_t)s + 1], 9 * sizeof(double));
    }
    return GAPGPU_OK;
}

int gapgpu_calc_lammps(gapgpu_context* c, int nlocal, int nghost, const int32_t* Z, int inum, const int32_t* ilist,
                       const int32_t* num_neigh, const int32_t* neigh, const double* lattice, const double* pos,
                       double* energy, double* local_e, double* virial, double* local_virial, double* force) {
    if (!c || nlocal < 0 || nghost < 0 || inum < 0 || !lattice || (nlocal + nghost > 0 && (!Z || !pos)) ||
        (inum > 0 && (!ilist || !num_neigh)))
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_lammps: bad argument");
    c->launches = 0;
    const int n = nlocal + nghost;
    if (nlocal == 0) {  // an empty region: every output zero, as the reference wrapper does
        if (energy) *energy = 0;
        if (virial) std::memset(virial, 0, 9 * sizeof(double));
        if (local_e) std::memset(local_e, 0, sizeof(double) * n);
        if (local_virial) std::memset(local_virial, 0, 9 * sizeof(double) * n);
        if (force) std::memset(force, 0, 3 * sizeof(double) * n);
        return GAPGPU_OK;
    }
    // the local atoms are the centres; the full per-local-atom lists are completed with
    // the ghost -> local entries so that ghosts receive their forces by the same gather
    std::vector<int32_t> local(n, 0);
    for (int k = 0; k < inum; ++k) {
        if (ilist[k] < 0 || ilist[k] >= n) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_lammps: ilist entry out of range");
        local[ilist[k]] = 1;
    }
    std::vector<int> cnt(n + 1, 0);
    long long total = 0;
    for (int k = 0; k < inum; ++k) total += num_neigh[k];
    if (total > 0 && !neigh) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_lammps: NULL neighbour list");
    for (long long q = 0, k = 0; k < inum; ++k)
        for (int m = 0; m < num_neigh[k]; ++m, ++q) {
            const int i = ilist[k], j = neigh[q] - 1;  // neighbours are 1-based, as quip_lammps_wrapper reads them
            if (j < 0 || j >= n || j == i) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_calc_lammps: neighbour index out of range");
            cnt[i + 1]++;
            if (!local[j]) cnt[j + 1]++;
        }
    for (int a = 0; a < n; ++a) cnt[a + 1] += cnt[a];
    std::vector<int> off(cnt), nj(cnt[n]), fill(cnt.begin(), cnt.end() - 1);
    for (long long q = 0, k = 0; k < inum; ++k)
        for (int m = 0; m < num_neigh[k]; ++m, ++q) {
            const int i = ilist[k], j = neigh[q] - 1;
            nj[fill[i]++] = j;
            if (!local[j]) nj[fill[j]++] = i;
        }
    int rc;
    if ((rc = copy_inputs(*c, n, pos, Z, local.data(), cudaMemcpyHostToDevice))) return rc;
    const int* dmask = c->mask.as<int>();
    const int prec = c->precision;
    if ((rc = load_external_neighbours(*c, n, off, nj, lattice, prec != GAPGPU_FP64))) return rc;
    const int pbc[3] = {0, 0, 0};
    if ((rc = prepare(*c, 1, &n, lattice, pbc, dmask, c->model->cutoff, LIST_GIVEN, prec))) return rc;
    apply_call_opts(*c, ArgOpts{});
    if ((rc = run_evaluation(*c, prec, dmask))) return rc;
    c->epc_valid = c->want_epc;
    double red[10];
    GG_CUDA(cudaMemcpyAsync(red, c->out_e.p, sizeof red, cudaMemcpyDeviceToHost, c->stream));
    if (force) GG_CUDA(cudaMemcpyAsync(force, c->out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c->stream));
    if (local_e) GG_CUDA(cudaMemcpyAsync(local_e, c->out_le.p, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
    if (local_virial)
        GG_CUDA(cudaMemcpyAsync(local_virial, c->out_lv.p, sizeof(double) * 9 * n, cudaMemcpyDeviceToHost, c->stream));
    GG_CUDA(cudaStreamSynchronize(c->stream));
    if ((rc = check_device_flags(*c))) return rc;
    if (energy) *energy = red[0];
    if (virial) std::memcpy(virial, red + 1, 9 * sizeof(double));
    return GAPGPU_OK;
}

int gapgpu_neighbours(gapgpu_context* c, int n, const double* pos, const double* lattice, const int32_t* pbc, double cutoff,
                      int32_t* offsets, int32_t* nbr_j, int32_t* nbr_shift, int64_t capacity, int64_t* total) {
    if (!c || n <= 0 || !pos || !lattice || !pbc) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_neighbours: bad argument");
    int rc;
    if ((rc = c->pos.ensure(sizeof(double) * 3 * n))) return rc;
    GG_CUDA(cudaMemcpyAsync(c->pos.p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice, c->stream));
    if ((rc = build_neighbours(*c, n, c->pos.as<double>(), lattice, pbc, cutoff, nullptr))) return rc;
    c->n_total = -1;  // the kept list is not an evaluation's list any more
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

int gapgpu_context_neighbours(gapgpu_context* c, int32_t* offsets, int32_t* nbr_j, int32_t* nbr_shift, double* nbr_r,
                              int64_t capacity, int64_t* total) {
    if (!c || !total) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_context_neighbours: NULL argument");
    if (c->n_total <= 0) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_context_neighbours: the context holds no evaluation's list");
    const int n = c->n_total;
    const long long P = c->n_pairs;
    GG_CUDA(cudaStreamSynchronize(c->stream));
    *total = P;
    if (offsets) GG_CUDA(cudaMemcpy(offsets, c->nbr_off.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    if (capacity < P || P == 0) return GAPGPU_OK;
    if (nbr_j) GG_CUDA(cudaMemcpy(nbr_j, c->nbr_j.p, sizeof(int) * P, cudaMemcpyDeviceToHost));
    if (nbr_shift) {
        std::vector<int> packed(P);
        GG_CUDA(cudaMemcpy(packed.data(), c->nbr_s.p, sizeof(int) * P, cudaMemcpyDeviceToHost));
        for (long long p = 0; p < P; ++p) {
            const int sh = packed[p];
            nbr_shift[3 * p] = (sh & 1023) - 512;
            nbr_shift[3 * p + 1] = ((sh >> 10) & 1023) - 512;
            nbr_shift[3 * p + 2] = ((sh >> 20) & 1023) - 512;
        }
    }
    if (nbr_r) {
        std::vector<double4> d(P);
        GG_CUDA(cudaMemcpy(d.data(), c->nbr_d.p, sizeof(double4) * P, cudaMemcpyDeviceToHost));
        for (long long p = 0; p < P; ++p) nbr_r[p] = d[p].w;
    }
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
    if ((rc = copy_inputs(*c, n, pos, Z, nullptr, cudaMemcpyHostToDevice))) return rc;
    if ((rc = build_neighbours(*c, n, c->pos.as<double>(), lattice, pbc, co.cutoff(), nullptr))) return rc;
    c->n_total = -1;  // the kept list is not an evaluation's list any more
    int nc = 0;
    if ((rc = c->centres.ensure(sizeof(int) * n))) return rc;
    c->cur_centres = c->centres.as<int>();
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
    gapgpu_context& cc = const_cast<gapgpu_context&>(*c);
    compute_timings(cc);
    const Timings& t = cc.t;
    double v[7] = {t.neighbours, t.soap_fwd, t.gemm, t.soap_bwd, t.pair2b, t.reduce, t.total};
    int k = std::min(capacity, 7);
    for (int i = 0; i < k; ++i) ms[i] = v[i];
    return k;
}

int gapgpu_probe_fp32_rate(gapgpu_context* c, double* tflops) {
    if (!c || !tflops) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_probe_fp32_rate: NULL argument");
    int rc, dev = 0, sms = 0;
    GG_CUDA(cudaGetDevice(&dev));
    GG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = 4 * sms, threads = 512, iters = 1 << 16;
    if ((rc = c->scratch.ensure(sizeof(float) * blocks))) return rc;
    cudaEvent_t e0, e1;
    GG_CUDA(cudaEventCreate(&e0));
    GG_CUDA(cudaEventCreate(&e1));
    double best = 0;
    for (int packed = 0; packed < 2; ++packed) {
        for (int rep = 0; rep < 3; ++rep) {  // the first launch of each form is a warm-up
            cudaEventRecord(e0, c->stream);
            if (packed) k_fma_rate<true><<<blocks, threads, 0, c->stream>>>(iters, 1.0f, c->scratch.as<float>());
            else k_fma_rate<false><<<blocks, threads, 0, c->stream>>>(iters, 1.0f, c->scratch.as<float>());
            cudaEventRecord(e1, c->stream);
            cudaError_t e = cudaEventSynchronize(e1);
            if (e != cudaSuccess) {
                cudaEventDestroy(e0);
                cudaEventDestroy(e1);
                GG_FAIL(GAPGPU_ERR_CUDA, std::string("gapgpu_probe_fp32_rate: ") + cudaGetErrorString(e));
            }
            float ms = 0;
            cudaEventElapsedTime(&ms, e0, e1);
            const double flops = 2.0 * FMA_CHAINS * (double)iters * blocks * threads;
            if (rep > 0 && ms > 0) best = std::max(best, flops / (ms * 1e-3) / 1e12);
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *tflops = best;
    return GAPGPU_OK;
}

int gapgpu_context_launches(const gapgpu_context* c, int64_t* launches) {
    if (!c || !launches) GG_FAIL(GAPGPU_ERR_ARG, "NULL argument");
    *launches = c->launches;
    return GAPGPU_OK;
}

}  // extern "C"
