// md.cu -- device-resident velocity-Verlet molecular dynamics of many replicas.
//
// Restates DynamicalSystem's advance_verlet1 / advance_verlet2
// (src/libAtoms/DynamicalSystem.f95:1814-2132, :2159-2383) as driven by
// DynamicalSystem_run (src/Potentials/Potential.f95:2304-2370):
//   advance_verlet1:  v += (dt/2) f/m ;  r += dt v
//   calc:             f = F(r)  (the GAP pipeline, all replicas in one batch)
//   advance_verlet2:  v += (dt/2) f/m
// with QUIP's skin rule for the connection (Connection.f95:1086-1125): the list is
// built at cutoff + skin and kept while the largest displacement since the build is
// below skin/2; otherwise only the pair displacements are refreshed
// (connection_calc_dists, :1321-1445).  Positions, velocities, forces and the
// neighbour lists never leave the GPU between steps.  Steps that keep the list replay
// the evaluation phase from a CUDA graph.
#include <cstring>
#include <vector>

#include "context.h"

struct gapgpu_md {
    gapgpu_context* ctx = nullptr;
    int nstruct = 0, n = 0;
    std::vector<int> n_atoms;
    std::vector<double> lattices;
    std::vector<int> pbcs;
    double dt = 1.0, skin = 0.0;
    gapgpu::DBuf velo, mass, ref;
    long long steps = 0, rebuilds = 0;
};

namespace gapgpu {
namespace {

__global__ void k_verlet1(int n, double* __restrict__ pos, double* __restrict__ velo, const double* __restrict__ f,
                          const double* __restrict__ mass, double dt) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double h = 0.5 * dt / mass[a];
    for (int k = 0; k < 3; ++k) {
        const double v = velo[3 * a + k] + h * f[3 * a + k];
        velo[3 * a + k] = v;
        pos[3 * a + k] += dt * v;
    }
}

__global__ void k_verlet2(int n, double* __restrict__ velo, const double* __restrict__ f, const double* __restrict__ mass,
                          double dt) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double h = 0.5 * dt / mass[a];
    for (int k = 0; k < 3; ++k) velo[3 * a + k] += h * f[3 * a + k];
}

// Neighbour list for the current positions: rebuilt at cutoff + skin when forced or
// when an atom has moved skin/2 or more since the last build, refreshed otherwise.
int connect(gapgpu_md& md, bool force_rebuild) {
    gapgpu_context& c = *md.ctx;
    int rc;
    bool rebuild = force_rebuild || md.skin <= 0.0;
    if (!rebuild) {
        double disp = 0;
        if ((rc = max_displacement(c, c.pos.as<double>(), md.ref.as<double>(), md.n, &disp))) return rc;
        rebuild = disp >= 0.5 * md.skin;
    }
    if ((rc = prepare(c, md.nstruct, md.n_atoms.data(), md.lattices.data(), md.pbcs.data(), nullptr,
                      c.model->cutoff + md.skin, rebuild ? LIST_BUILD : LIST_REFRESH, c.precision)))
        return rc;
    if (rebuild) {
        GG_CUDA(cudaMemcpyAsync(md.ref.p, c.pos.p, sizeof(double) * 3 * md.n, cudaMemcpyDeviceToDevice, c.stream));
        md.rebuilds++;
    }
    return GAPGPU_OK;
}

}  // namespace
}  // namespace gapgpu

using namespace gapgpu;

extern "C" {

int gapgpu_md_create(const gapgpu_model* model, int precision, int nstruct, const int32_t* n_atoms, const double* pos,
                     const double* velo, const double* mass, const int32_t* Z, const double* lattices, const int32_t* pbcs,
                     double dt, double skin, gapgpu_md** out) {
    if (!model || !out || nstruct < 1 || !n_atoms || !pos || !velo || !mass || !Z || !lattices || !pbcs || !(dt > 0) ||
        !(skin >= 0))
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_md_create: bad argument");
    *out = nullptr;
    long long n = 0;
    for (int s = 0; s < nstruct; ++s) {
        if (n_atoms[s] <= 0) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_md_create: every replica needs atoms");
        n += n_atoms[s];
    }
    if (n > (1LL << 30)) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_md_create: too many atoms");
    gapgpu_context* ctx = nullptr;
    int rc;
    if ((rc = gapgpu_context_create(model, precision, &ctx))) return rc;
    gapgpu_md* md = new gapgpu_md();
    md->ctx = ctx;
    ctx->graph_mode = 1;
    ctx->timed = false;
    md->nstruct = nstruct;
    md->n = (int)n;
    md->n_atoms.assign(n_atoms, n_atoms + nstruct);
    md->lattices.assign(lattices, lattices + 9 * (size_t)nstruct);
    md->pbcs.assign(pbcs, pbcs + 3 * (size_t)nstruct);
    md->dt = dt;
    md->skin = skin;
    auto fail = [&](int code) {
        gapgpu_md_destroy(md);
        return code;
    };
    gapgpu_context& c = *ctx;
    if ((rc = c.pos.ensure(sizeof(double) * 3 * n)) || (rc = c.Z.ensure(sizeof(int) * n)) ||
        (rc = md->velo.ensure(sizeof(double) * 3 * n)) || (rc = md->mass.ensure(sizeof(double) * n)) ||
        (rc = md->ref.ensure(sizeof(double) * 3 * n)))
        return fail(rc);
    cudaError_t e;
    if ((e = cudaMemcpy(c.pos.p, pos, sizeof(double) * 3 * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(c.Z.p, Z, sizeof(int) * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(md->velo.p, velo, sizeof(double) * 3 * n, cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(md->mass.p, mass, sizeof(double) * n, cudaMemcpyHostToDevice)) != cudaSuccess) {
        set_error(std::string("gapgpu_md_create: ") + cudaGetErrorString(e));
        return fail(GAPGPU_ERR_CUDA);
    }
    // forces at t = 0 (the first advance_verlet1 needs them)
    if ((rc = connect(*md, true)) || (rc = run_evaluation(c, c.precision, nullptr))) return fail(rc);
    GG_CUDA(cudaStreamSynchronize(c.stream));
    if ((rc = check_device_flags(c))) return fail(rc);
    *out = md;
    return GAPGPU_OK;
}

int gapgpu_md_step(gapgpu_md* md, int nsteps) {
    if (!md || nsteps < 0) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_md_step: bad argument");
    gapgpu_context& c = *md->ctx;
    c.launches = 0;
    const int TB = 256, nb = (md->n + TB - 1) / TB;
    int rc;
    for (int k = 0; k < nsteps; ++k) {
        k_verlet1<<<nb, TB, 0, c.stream>>>(md->n, c.pos.as<double>(), md->velo.as<double>(), c.out_f.as<double>(),
                                           md->mass.as<double>(), md->dt);
        c.launches++;
        if ((rc = connect(*md, false))) return rc;
        if ((rc = run_evaluation(c, c.precision, nullptr))) return rc;
        k_verlet2<<<nb, TB, 0, c.stream>>>(md->n, md->velo.as<double>(), c.out_f.as<double>(), md->mass.as<double>(),
                                           md->dt);
        c.launches++;
        md->steps++;
    }
    GG_CUDA(cudaGetLastError());
    GG_CUDA(cudaStreamSynchronize(c.stream));
    return check_device_flags(c);
}

int gapgpu_md_state(gapgpu_md* md, double* pos, double* velo, double* force, double* energies, double* virials) {
    if (!md) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_md_state: NULL handle");
    gapgpu_context& c = *md->ctx;
    const size_t n = md->n;
    std::vector<double> red(10 * (size_t)md->nstruct);
    if (pos) GG_CUDA(cudaMemcpyAsync(pos, c.pos.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.stream));
    if (velo) GG_CUDA(cudaMemcpyAsync(velo, md->velo.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.stream));
    if (force) GG_CUDA(cudaMemcpyAsync(force, c.out_f.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, c.stream));
    GG_CUDA(cudaMemcpyAsync(red.data(), c.out_e.p, sizeof(double) * red.size(), cudaMemcpyDeviceToHost, c.stream));
    GG_CUDA(cudaStreamSynchronize(c.stream));
    for (int s = 0; s < md->nstruct; ++s) {
        if (energies) energies[s] = red[10 * (size_t)s];
        if (virials) std::memcpy(virials + 9 * (size_t)s, &red[10 * (size_t)s + 1], 9 * sizeof(double));
    }
    return GAPGPU_OK;
}

int gapgpu_md_counters(const gapgpu_md* md, int64_t* steps, int64_t* rebuilds, int64_t* graph_replays) {
    if (!md) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_md_counters: NULL handle");
    if (steps) *steps = md->steps;
    if (rebuilds) *rebuilds = md->rebuilds;
    if (graph_replays) *graph_replays = md->ctx->graph_hits;
    return GAPGPU_OK;
}

gapgpu_context* gapgpu_md_context(gapgpu_md* md) { return md ? md->ctx : nullptr; }

void gapgpu_md_destroy(gapgpu_md* md) {
    if (!md) return;
    md->velo.release();
    md->mass.release();
    md->ref.release();
    gapgpu_context_destroy(md->ctx);
    delete md;
}

}  // extern "C"
