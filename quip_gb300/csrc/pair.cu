// pair.cu -- K6 distance_2b + ard_se GP, and K7/K8: deterministic force / virial /
// energy assembly.
//
// distance_2b (GAP descriptors_module, absent; pinned by tests/test_gappot.py): one
// descriptor per DIRECTED pair (i -> j, r < cutoff, species (Z1,Z2) in either order),
// value r, covariance_cutoff fc(r), energy split e fc / 2 to i and j.
// ard_se: e = sum_s alpha_s delta^2 sc_s exp(-(r - x_s)^2 / (2 theta^2)).
//
// Assembly (src/Potentials/IPModel_GAP.f95:472-499, :523-596): every descriptor
// contributes, per directed pair p = (i -> j, d = r_j + L s - r_i), a vector
// f_p = dE_i / dr_j.  The reference scatters F(j) -= f_p, F(i) += f_p and
// virial(j) -= d (x) f_p.  Here each atom GATHERS over its own list using the
// reverse-pair index (the pair j -> i of p is rev[p], with d_rev = -d), so there are
// no floating-point atomics and the result is bit-identical run to run:
//   F_a   = sum_{p in a} (f_p - f_rev(p))
//   W_a   = sum_{p in a} d_p (x) f_rev(p)
//   e_a   = eatom_a + sum_{p in a} (epair_p + epair_rev(p)) + e0(Z_a) [mask]
#include <algorithm>
#include <vector>

#include "context.h"

namespace gapgpu {
namespace {

__device__ __forceinline__ double fcos(double x) { return cos(x); }
__device__ __forceinline__ float fcos(float x) { return cosf(x); }
__device__ __forceinline__ double fsin(double x) { return sin(x); }
__device__ __forceinline__ float fsin(float x) { return sinf(x); }

template <class R>
__device__ __forceinline__ void fcut(R r, R rc, R w, R& f, R& df) {
    if (r > rc) { f = 0; df = 0; return; }
    if (r > rc - w) {
        const R pi = (R)3.14159265358979323846;
        R a = pi * (r - rc + w) / w;
        f = (R)0.5 * (fcos(a) + (R)1);
        df = -(R)0.5 * pi * fsin(a) / w;
        return;
    }
    f = 1; df = 0;
}

// The distance_2b coordinates of a model, evaluated together in one pass over the pairs.
constexpr int MAX_2B = 16;
struct Pair2bSet {
    int n;
    struct Entry {
        double rc, w, it2;      // cutoff, transition width, 1 / theta^2
        int Z1, Z2, M;
        const void* X;          // [M] sparse points (R)
        const void* coef;       // [M] alpha sparseCutoff delta^2 (R)
    } c[MAX_2B];
};

// All distance_2b coordinates of the set in one pass; every fpair/epair slot has exactly
// one writer.
//   FP64 (FP64 exp is the cost): one thread per canonical directed pair (i < j, or
//   i == j with the shift lexicographically positive) writes its own slot and, with the
//   opposite force, its reverse pair's: both have the same r and descriptor value.
//   FP32: one thread per directed pair writes only its own slot, from its own staged
//   displacement (the neighbour build forms d(b->a) = -d(a->b) with sign-symmetric
//   round-to-nearest steps), so the slots are written in order, without the scattered
//   read-modify-write of the reverse slot, for twice the (cheap) FP32 exp work.
// exp of the GP kernel terms: the FP64 path's exp, the fast intrinsic in the FP32 path
// (relative error ~1e-6 at its arguments, below the FP32 path's other rounding)
__device__ __forceinline__ double exp_gp(double x) { return exp(x); }
__device__ __forceinline__ float exp_gp(float x) { return __expf(x); }

template <class R>
__global__ void k_pair_2b(long long P, const int* __restrict__ Z, const int* __restrict__ mask, const int* __restrict__ ni,
                          const int* __restrict__ nj, const int* __restrict__ ns, const int* __restrict__ rev,
                          const double4* __restrict__ nd, const Pair2bSet set, double* __restrict__ fpair,
                          double* __restrict__ epair) {
    constexpr bool OWN = sizeof(R) == 4;
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int a = ni[p], b = nj[p];
    const bool ca = !mask || mask[a], cb = !OWN && (!mask || mask[b]);
    if (OWN) {
        if (!ca) return;
    } else {
        if (a > b) return;
        if (a == b) {
            int s = ns[p];
            int s0 = (s & 1023) - 512, s1 = ((s >> 10) & 1023) - 512, s2 = ((s >> 20) & 1023) - 512;
            if (!(s0 > 0 || (s0 == 0 && (s1 > 0 || (s1 == 0 && s2 > 0))))) return;
        }
        if (!ca && !cb) return;
    }
    const double4 d = nd[p];
    const int za = Z[a], zb = Z[b];
    // FP64 path: every step in double; mixed path: FP32 GP sums and force, FP64 accumulation.
    const R r = (R)d.w;
    R g = 0, ef = 0;
    bool any = false;
    for (int k = 0; k < set.n; ++k) {
        const Pair2bSet::Entry& cd = set.c[k];
        if (d.w >= cd.rc) continue;
        const bool zi1 = cd.Z1 == 0 || za == cd.Z1, zj2 = cd.Z2 == 0 || zb == cd.Z2;
        const bool zi2 = cd.Z2 == 0 || za == cd.Z2, zj1 = cd.Z1 == 0 || zb == cd.Z1;
        if (!((zi1 && zj2) || (zi2 && zj1))) continue;
        const R* X = static_cast<const R*>(cd.X);
        const R* coef = static_cast<const R*>(cd.coef);
        const R it2 = (R)cd.it2;
        R e = 0, de = 0;
        for (int s = 0; s < cd.M; ++s) {
            const R t = r - X[s];
            const R kv = coef[s] * exp_gp(-(R)0.5 * t * t * it2);
            e += kv;
            de -= kv * t * it2;
        }
        R f, df;
        fcut<R>(r, (R)cd.rc, (R)cd.w, f, df);
        g += de * f + e * df;
        ef += e * f;
        any = true;
    }
    if (!any) return;
    const R ir = (R)1 / r;
    const double fx = (double)(g * (R)d.x * ir), fy = (double)(g * (R)d.y * ir), fz = (double)(g * (R)d.z * ir);
    const double h = (double)((R)0.5 * ef);
    if (ca) {
        fpair[3 * (size_t)p] += fx; fpair[3 * (size_t)p + 1] += fy; fpair[3 * (size_t)p + 2] += fz;
        epair[p] += h;
    }
    if (cb) {
        const long long q = rev[p];
        fpair[3 * (size_t)q] -= fx; fpair[3 * (size_t)q + 1] -= fy; fpair[3 * (size_t)q + 2] -= fz;
        epair[q] += h;
    }
}

// GATHER_LANES lanes per atom: lane k takes the atom's pairs k, k + GATHER_LANES, ... in
// order, and the lanes' sums are combined by an xor butterfly (the same fixed order, and
// the same bits, in every lane); lane 0 writes.  Deterministic: no atomics.
constexpr int GATHER_LANES = 4;
__global__ void k_gather(int n, const int* __restrict__ Z, const int* __restrict__ mask, const int* __restrict__ off,
                         const int* __restrict__ rev, const double4* __restrict__ nd, const double* __restrict__ fpair,
                         const double* __restrict__ epair, const double* __restrict__ eatom, const double* __restrict__ e0,
                         double escale, double* __restrict__ le, double* __restrict__ F, double* __restrict__ LV) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x, a = g / GATHER_LANES, sub = g % GATHER_LANES;
    const bool ok = a < n;  // lanes past the last atom still take part in the butterfly
    double f0 = 0, f1 = 0, f2 = 0, e = 0;
    double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int p0 = ok ? off[a] : 0, p1 = ok ? off[a + 1] : 0;
    for (int p = p0 + sub; p < p1; p += GATHER_LANES) {
        int q = rev[p];
        double4 d = nd[p];
        double g0 = fpair[3 * (size_t)q], g1 = fpair[3 * (size_t)q + 1], g2 = fpair[3 * (size_t)q + 2];
        f0 += fpair[3 * (size_t)p] - g0;
        f1 += fpair[3 * (size_t)p + 1] - g1;
        f2 += fpair[3 * (size_t)p + 2] - g2;
        // virial_a(r, c) -= (-d)(r) f_rev(c)   (column-major 3x3)
        double dd[3] = {d.x, d.y, d.z}, gg[3] = {g0, g1, g2};
#pragma unroll
        for (int cc = 0; cc < 3; ++cc)
#pragma unroll
            for (int r = 0; r < 3; ++r) v[3 * cc + r] += dd[r] * gg[cc];
        e += epair[p] + epair[q];
    }
#pragma unroll
    for (int o = 1; o < GATHER_LANES; o <<= 1) {
        f0 += __shfl_xor_sync(0xffffffffu, f0, o);
        f1 += __shfl_xor_sync(0xffffffffu, f1, o);
        f2 += __shfl_xor_sync(0xffffffffu, f2, o);
        e += __shfl_xor_sync(0xffffffffu, e, o);
#pragma unroll
        for (int k = 0; k < 9; ++k) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
    }
    if (!ok || sub != 0) return;
    e += eatom[a];
    if (!mask || mask[a]) {
        int z = Z[a];
        e += (z >= 0 && z < 128) ? e0[z] : 0.0;
    }
    le[a] = escale * e;
    F[3 * (size_t)a] = escale * f0;
    F[3 * (size_t)a + 1] = escale * f1;
    F[3 * (size_t)a + 2] = escale * f2;
    for (int k = 0; k < 9; ++k) LV[9 * (size_t)a + k] = escale * v[k];
}

// Deterministic per-structure sums E_s = sum le, virial_s = sum LV in two fixed-order
// levels: chunk k (atoms chunk[k].x .. chunk[k].y - 1 of one structure, RED_CHUNK at a
// time from the structure's first atom) is reduced by one block into part[k][10]; then
// one block per structure sums its chunks in order.  The arithmetic of a structure does
// not depend on where it sits in a batch, so a structure gives the same bits alone and
// batched, run after run (no atomics).
constexpr int RED_THREADS = 256;

__device__ __forceinline__ void block_sum10(double (&acc)[10], double (*sh)[RED_THREADS]) {
    for (int k = 0; k < 10; ++k) sh[k][threadIdx.x] = acc[k];
    __syncthreads();
    for (int s = RED_THREADS / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int k = 0; k < 10; ++k) sh[k][threadIdx.x] += sh[k][threadIdx.x + s];
        __syncthreads();
    }
}

__global__ void __launch_bounds__(RED_THREADS) k_reduce_part(const int2* __restrict__ chunk, const double* __restrict__ le,
                                                             const double* __restrict__ LV, double* __restrict__ part) {
    __shared__ double sh[10][RED_THREADS];
    double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    const int2 ch = chunk[blockIdx.x];
    for (int a = ch.x + threadIdx.x; a < ch.y; a += RED_THREADS) {
        acc[0] += le[a];
        for (int k = 0; k < 9; ++k) acc[1 + k] += LV[9 * (size_t)a + k];
    }
    block_sum10(acc, sh);
    if (threadIdx.x < 10) part[10 * (size_t)blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

__global__ void __launch_bounds__(RED_THREADS) k_reduce_final(const int* __restrict__ schunk, const double* __restrict__ part,
                                                              double* __restrict__ out) {
    __shared__ double sh[10][RED_THREADS];
    double acc[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int b = schunk[blockIdx.x] + threadIdx.x; b < schunk[blockIdx.x + 1]; b += RED_THREADS)
        for (int k = 0; k < 10; ++k) acc[k] += part[10 * (size_t)b + k];
    block_sum10(acc, sh);
    if (threadIdx.x < 10) out[10 * (size_t)blockIdx.x + threadIdx.x] = sh[threadIdx.x][0];
}

// energy_per_coordinate of one distance_2b coordinate: per canonical pair, e fc times the
// number of its two directed instances whose centre is evaluated (instance i -> j is in
// the sum when atom i is in the mask); 0 in every other pair slot.
template <class R>
__global__ void k_pair_2b_energy(long long P, const int* __restrict__ Z, const int* __restrict__ mask,
                                 const int* __restrict__ ni, const int* __restrict__ nj, const int* __restrict__ ns,
                                 const double4* __restrict__ nd, const Pair2bSet::Entry cd, double* __restrict__ out) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P) return;
    double v = 0.0;
    const int a = ni[p], b = nj[p];
    bool canonical = a < b;
    if (a == b) {
        int s = ns[p];
        int s0 = (s & 1023) - 512, s1 = ((s >> 10) & 1023) - 512, s2 = ((s >> 20) & 1023) - 512;
        canonical = s0 > 0 || (s0 == 0 && (s1 > 0 || (s1 == 0 && s2 > 0)));
    }
    const double4 d = nd[p];
    if (canonical && d.w < cd.rc) {
        const int za = Z[a], zb = Z[b];
        const bool zi1 = cd.Z1 == 0 || za == cd.Z1, zj2 = cd.Z2 == 0 || zb == cd.Z2;
        const bool zi2 = cd.Z2 == 0 || za == cd.Z2, zj1 = cd.Z1 == 0 || zb == cd.Z1;
        const int w = (!mask || mask[a] ? 1 : 0) + (!mask || mask[b] ? 1 : 0);
        if (((zi1 && zj2) || (zi2 && zj1)) && w > 0) {
            const R* X = static_cast<const R*>(cd.X);
            const R* coef = static_cast<const R*>(cd.coef);
            const R r = (R)d.w, it2 = (R)cd.it2;
            R e = 0;
            for (int s = 0; s < cd.M; ++s) {
                const R t = r - X[s];
                e += coef[s] * exp(-(R)0.5 * t * t * it2);
            }
            R f, df;
            fcut<R>(r, (R)cd.rc, (R)cd.w, f, df);
            v = (double)w * (double)(e * f);
        }
    }
    out[p] = v;
}

__global__ void k_scatter_centres(int nc, const int* __restrict__ centres, const double* __restrict__ ecent,
                                  double* __restrict__ ea) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nc) ea[centres[i]] = ecent[i];
}

// One block per structure: the sum of vals over the structure's atoms (off == NULL) or its
// pair slots (the CSR rows of its atoms), in a fixed order -> out[s * ncoord + k].
__global__ void __launch_bounds__(RED_THREADS) k_epc_reduce(const double* __restrict__ vals,
                                                           const GeomDev* __restrict__ geoms, const int* __restrict__ off,
                                                           int ncoord, int k, double* __restrict__ out) {
    __shared__ double sh[RED_THREADS];
    const GeomDev& g = geoms[blockIdx.x];
    const long long b = off ? off[g.atom_begin] : g.atom_begin, e = off ? off[g.atom_end] : g.atom_end;
    double acc = 0.0;
    for (long long i = b + threadIdx.x; i < e; i += RED_THREADS) acc += vals[i];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int st = RED_THREADS / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[(size_t)blockIdx.x * ncoord + k] = sh[0];
}

}  // namespace

int epc_soap(gapgpu_context& c, int k, int nc, int n) {
    int rc;
    if ((rc = c.epca.ensure(sizeof(double) * (size_t)std::max(n, 1)))) return rc;
    GG_CUDA(cudaMemsetAsync(c.epca.p, 0, sizeof(double) * (size_t)n, c.stream));
    if (nc > 0)
        k_scatter_centres<<<(nc + 127) / 128, 128, 0, c.stream>>>(nc, c.cur_centres, c.ecent.as<double>(),
                                                                 c.epca.as<double>());
    k_epc_reduce<<<c.nstruct, RED_THREADS, 0, c.stream>>>(c.epca.as<double>(), c.geoms.as<GeomDev>(), nullptr,
                                                         (int)c.model->coords.size(), k, c.epc_out.as<double>());
    c.launches += nc > 0 ? 2 : 1;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

int epc_pair(gapgpu_context& c, const Coordinate& co, int k, const int* d_mask) {
    const long long P = c.n_pairs;
    if (P == 0) return GAPGPU_OK;  // no pairs: the zeroed output stands
    int rc;
    if ((rc = c.epcp.ensure(sizeof(double) * (size_t)P))) return rc;
    const bool fp64 = c.precision == GAPGPU_FP64;
    {
        Pair2bSet::Entry e{co.d2_rc, co.d2_w, 1.0 / (co.theta[0] * co.theta[0]), co.d2_Z1, co.d2_Z2, co.M,
                           fp64 ? (const void*)co.dX64 : (const void*)co.dXf32,
                           fp64 ? (const void*)co.dcoef : (const void*)co.dcoef32};
        const int TB = 256;
        const unsigned nb = (unsigned)((P + TB - 1) / TB);
        if (fp64)
            k_pair_2b_energy<double><<<nb, TB, 0, c.stream>>>(P, c.Z.as<int>(), d_mask, c.nbr_i.as<int>(),
                                                               c.nbr_j.as<int>(), c.nbr_s.as<int>(),
                                                               c.nbr_d.as<double4>(), e, c.epcp.as<double>());
        else
            k_pair_2b_energy<float><<<nb, TB, 0, c.stream>>>(P, c.Z.as<int>(), d_mask, c.nbr_i.as<int>(),
                                                              c.nbr_j.as<int>(), c.nbr_s.as<int>(),
                                                              c.nbr_d.as<double4>(), e, c.epcp.as<double>());
        c.launches++;
    }
    k_epc_reduce<<<c.nstruct, RED_THREADS, 0, c.stream>>>(c.epcp.as<double>(), c.geoms.as<GeomDev>(), c.nbr_off.as<int>(),
                                                         (int)c.model->coords.size(), k, c.epc_out.as<double>());
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

int pair_2b(gapgpu_context& c, const std::vector<const Coordinate*>& coords, const int* d_mask) {
    for (const Coordinate* co : coords)
        if (co->cov != COV_ARD_SE) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "distance_2b needs the ard_se covariance");
    const long long P = c.n_pairs;
    if (P == 0 || coords.empty()) return GAPGPU_OK;
    const bool fp64 = c.precision == GAPGPU_FP64;
    const int TB = 256;
    const unsigned nb = (unsigned)((P + TB - 1) / TB);
    for (size_t k0 = 0; k0 < coords.size(); k0 += MAX_2B) {
        Pair2bSet set{};
        set.n = (int)std::min<size_t>(MAX_2B, coords.size() - k0);
        for (int k = 0; k < set.n; ++k) {
            const Coordinate& co = *coords[k0 + k];
            Pair2bSet::Entry& e = set.c[k];
            e.rc = co.d2_rc;
            e.w = co.d2_w;
            e.it2 = 1.0 / (co.theta[0] * co.theta[0]);
            e.Z1 = co.d2_Z1;
            e.Z2 = co.d2_Z2;
            e.M = co.M;
            e.X = fp64 ? (const void*)co.dX64 : (const void*)co.dXf32;
            e.coef = fp64 ? (const void*)co.dcoef : (const void*)co.dcoef32;
        }
        if (fp64)
            k_pair_2b<double><<<nb, TB, 0, c.stream>>>(P, c.Z.as<int>(), d_mask, c.nbr_i.as<int>(), c.nbr_j.as<int>(),
                                                       c.nbr_s.as<int>(), c.nbr_rev.as<int>(), c.nbr_d.as<double4>(), set,
                                                       c.fpair.as<double>(), c.epair.as<double>());
        else
            k_pair_2b<float><<<nb, TB, 0, c.stream>>>(P, c.Z.as<int>(), d_mask, c.nbr_i.as<int>(), c.nbr_j.as<int>(),
                                                      c.nbr_s.as<int>(), c.nbr_rev.as<int>(), c.nbr_d.as<double4>(), set,
                                                      c.fpair.as<double>(), c.epair.as<double>());
        c.launches++;
        GG_CUDA(cudaGetLastError());
    }
    return GAPGPU_OK;
}

int gather_into(gapgpu_context& c, int n, const double* e0, double escale, double* le, double* F, double* LV) {
    const int TB = 128;
    k_gather<<<(unsigned)(((size_t)n * GATHER_LANES + TB - 1) / TB), TB, 0, c.stream>>>(n, c.Z.as<int>(), nullptr, c.nbr_off.as<int>(), c.nbr_rev.as<int>(),
                                                    c.nbr_d.as<double4>(), c.fpair.as<double>(), c.epair.as<double>(),
                                                    c.eatom.as<double>(), e0, escale, le, F, LV);
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

int gather_outputs(gapgpu_context& c, const gapgpu_model& m, int n, const int* d_mask) {
    const int nchunks = (int)c.h_chunks.size() / 2, ns = c.nstruct;
    const int TB = 128;
    k_gather<<<(unsigned)(((size_t)n * GATHER_LANES + TB - 1) / TB), TB, 0, c.stream>>>(n, c.Z.as<int>(), d_mask, c.nbr_off.as<int>(), c.nbr_rev.as<int>(),
                                                    c.nbr_d.as<double4>(), c.fpair.as<double>(), c.epair.as<double>(),
                                                    c.eatom.as<double>(), m.de0, m.E_scale, c.out_le.as<double>(),
                                                    c.out_f.as<double>(), c.out_lv.as<double>());
    k_reduce_part<<<nchunks, RED_THREADS, 0, c.stream>>>(c.chunks.as<int2>(), c.out_le.as<double>(), c.out_lv.as<double>(),
                                                        c.redpart.as<double>());
    k_reduce_final<<<ns, RED_THREADS, 0, c.stream>>>(c.schunk.as<int>(), c.redpart.as<double>(), c.out_e.as<double>());
    c.launches += 3;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

}  // namespace gapgpu
