// soap.cu -- K3/K4 SOAP expansion, power spectrum and normalisation (forward) and
// K4^T/K7 adjoint: dE/dq -> dE/dp -> dE/dc -> per-pair force contributions.
//
// The descriptor is GAP's `soap` (descriptors_module of the libAtoms/GAP submodule,
// absent from the reference checkout).  Its conventions were recovered from the
// reference's fixtures (tests/Si.soap.cur_points.json, tests/test_descriptor.py):
//   rho_j(r_b) collocation : exp(-alpha (r^2 + r_b^2)) i_l(2 alpha r r_b), written with
//                            exp(-alpha (r -+ r_b)^2) and the upward recurrence
//                            i_l = i_{l-2} - (2l-1)/x i_{l-1}
//   radial coefficients     : R_nl(r) = fc(r) sum_a rho_l(r, r_a) T_an
//   expansion               : c[s][n][lm] = sum_{j in species s, r_ij < rc} R_nl(r_ij) Y_lm(r^_ij)
//                            + central atom (l = 0, own species channel)
//   power spectrum          : p[(ia,jb<=ia), l] = sqrt2^(ia!=jb) / sqrt(2l+1) sum_m c_ia,lm c_jb,lm
//   descriptor              : q = p / |p|, q[dim-1] = covariance_sigma0
// Real orthonormal spherical harmonics replace GAP's complex ones; the power
// spectrum is invariant under that unitary change of basis.
//
// Gradients are never materialised as dq/dr (3*dim per pair).  The backward pass
// contracts dE/dq with the normalisation Jacobian (FP64), forms
// dE/dc[a][lm] = sum_b H_l[a][b] c[b][lm], and for each pair computes
// f_ij = dE_i/dr_j = sum_{n,lm} dE/dc[s_j][n][lm] d(R_nl Y_lm)/dr_j, which is exactly
// the reference's matmul(gradPredict, grad_data(:,:,n)) (IPModel_GAP.f95:479) for the
// neighbour entry n = j; the centre entry is minus the sum over neighbours.
#include <cub/cub.cuh>
#include <cuda_fp16.h>
#include <cmath>
#include <vector>
#include <climits>
#include <mutex>
#include "context.h"

namespace gapgpu {

namespace {

// Constant block of one SOAP coordinate in the working precision R, uploaded once per
// model and copied into shared memory by every block (offsets in elements of R):
//   T[a][n] orthonormalising transform (also as Tt[n][a] and Tp[a][n], zero-padded to
//   multiples of 4 for vector loads), rb[a] radial grid, cr[n] central-atom l = 0
//   term, lf[l] = 1/sqrt(2l+1), yn[l*l+m] Ylm normalisation (sqrt2 folded in for m > 0),
//   ra/rbb[l*l+m] Legendre recurrence P_lm = ra t P_(l-1)m - rbb P_(l-2)m (l >= m+2).
struct SoapTab {
    int T, Tt, Tp, rb, cr, lf, yn, ra, rbb, size;
};
__host__ __device__ __forceinline__ int nmp_of(int nm) { return (nm + 3) & ~3; }
__host__ __device__ __forceinline__ SoapTab soap_tab(int nm, int L) {
    SoapTab t;
    int o = 0;
    const int NMP = nmp_of(nm);
    t.T = o; o += nm * nm;
    o = (o + 3) & ~3;
    t.Tt = o; o += nm * NMP;   // Tt[n][a] = T[a][n], rows zero-padded to NMP
    t.Tp = o; o += NMP * NMP;  // Tp[a][n] = T[a][n], zero-padded to NMP x NMP
    t.rb = o; o += nm;
    t.cr = o; o += nm;
    t.lf = o; o += L;
    t.yn = o; o += L * L;
    t.ra = o; o += L * L;
    t.rbb = o; o += L * L;
    t.size = (o + 7) & ~7;  // keeps what follows 32-byte aligned for R = double
    return t;
}

template <class R>
struct alignas(4 * sizeof(R)) Dual {  // a value and three derivatives
    R v, x, y, z;
};
__device__ __forceinline__ double rexp(double x) { return exp(x); }
__device__ __forceinline__ float rexp(float x) { return __expf(x); }
__device__ __forceinline__ double rcos(double x) { return cos(x); }
__device__ __forceinline__ float rcos(float x) { return cosf(x); }
__device__ __forceinline__ double rsin(double x) { return sin(x); }
__device__ __forceinline__ float rsin(float x) { return sinf(x); }
__device__ __forceinline__ double rinv(double x) { return 1.0 / x; }
__device__ __forceinline__ float rinv(float x) { return __frcp_rn(x); }

// coordination_function and its derivative
template <class R>
__device__ __forceinline__ void cutoff_fn(R r, R rc, R w, R& f, R& df) {
    if (r > rc) { f = 0; df = 0; return; }
    if (r > rc - w) {
        const R pi = (R)3.14159265358979323846;
        R a = pi * (r - rc + w) / w;
        f = (R)0.5 * (rcos(a) + (R)1);
        df = -(R)0.5 * pi * rsin(a) / w;
        return;
    }
    f = 1; df = 0;
}

// Column m of the real spherical harmonics Y_lm(u), l = m..L-1, written to
// Y[l*l + l +- m] for the unit vector u; (cm + i sm) = (ux + i uy)^m.
template <class R>
__device__ void ylm_column(int m, int L, R xr, R yr, R t, const R* __restrict__ K, const SoapTab& tb, R* Y) {
    R cm = 1, sm = 0;
    for (int k = 0; k < m; ++k) {
        R c2 = cm * xr - sm * yr;
        sm = sm * xr + cm * yr;
        cm = c2;
    }
    R qmm = 1;
    for (int k = 1; k <= 2 * m - 1; k += 2) qmm *= (R)k;
    R q2 = 0, q1 = 0;
    for (int l = m; l < L; ++l) {
        const int i = l * l + m;
        R q;
        if (l == m) q = qmm;
        else if (l == m + 1) q = (R)(2 * m + 1) * t * qmm;
        else q = K[tb.ra + i] * t * q1 - K[tb.rbb + i] * q2;
        q2 = q1;
        q1 = q;
        const R nrm = K[tb.yn + i];
        if (m == 0) Y[l * l + l] = nrm * q;
        else {
            Y[l * l + l + m] = nrm * q * cm;
            Y[l * l + l - m] = nrm * q * sm;
        }
    }
}

// Same column with the gradient of its Cartesian form N_lm Q_lm(u_z) Re/Im (u_x + i u_y)^m
// with respect to the components of u taken as independent: d/du_x (u_x + i u_y)^m =
// m (u_x + i u_y)^(m-1), d/du_y = i m (u_x + i u_y)^(m-1), and Q'_lm follows Q_lm's
// recurrence.  Y[lm] = (Y, dY/du_x, dY/du_y, dY/du_z); the tangential projection
// (I - u u^T) / r is applied once per neighbour after the contraction.
template <class R>
__device__ void ylm_column_cart(int m, int L, R xr, R yr, R zr, const R* __restrict__ K, const SoapTab& tb,
                                Dual<R>* Y) {
    R cm = 1, sm = 0, cp = 1, sp = 0;  // (u_x + i u_y)^m and ^(m-1)
    for (int k = 0; k < m; ++k) {
        cp = cm;
        sp = sm;
        const R c2 = cm * xr - sm * yr;
        sm = sm * xr + cm * yr;
        cm = c2;
    }
    R qmm = 1;
    for (int k = 1; k <= 2 * m - 1; k += 2) qmm *= (R)k;
    R q1 = 0, q2 = 0, d1 = 0, d2 = 0;
    const R fm = (R)m;
    for (int l = m; l < L; ++l) {
        const int i = l * l + m;
        R q, d;
        if (l == m) {
            q = qmm;
            d = 0;
        } else if (l == m + 1) {
            q = (R)(2 * m + 1) * zr * qmm;
            d = (R)(2 * m + 1) * qmm;
        } else {
            const R ra = K[tb.ra + i], rb = K[tb.rbb + i];
            q = ra * zr * q1 - rb * q2;
            d = ra * (q1 + zr * d1) - rb * d2;
        }
        q2 = q1;
        q1 = q;
        d2 = d1;
        d1 = d;
        const R nrm = K[tb.yn + i];
        const R nq = nrm * q, nd = nrm * d;
        if (m == 0) Y[l * l + l] = {nq, (R)0, (R)0, nd};
        else {
            const R a = nq * fm;
            Y[l * l + l + m] = {nq * cm, a * cp, -a * sp, nd * cm};
            Y[l * l + l - m] = {nq * sm, a * sp, a * cp, nd * sm};
        }
    }
}

// scale * rho_l(r, r_b) -> out[l * stride] for l = 0..L-1 and (when dout is given)
// d rho_l / dr -> dout[l * stride], with the upward recurrence carried in registers.
template <class R>
__device__ void radial_collocation(R r, R rb, R alpha, int L, R scale, R* out, R* dout, int stride) {
    if (rb == (R)0) {
        const R e = rexp(-alpha * r * r);
        out[0] = scale * e;
        if (dout) dout[0] = -(R)2 * alpha * r * e;
        for (int l = 1; l < L; ++l) { out[l * stride] = 0; if (dout) dout[l * stride] = 0; }
        return;
    }
    const R x = (R)2 * alpha * r * rb;
    const R em = rexp(-alpha * (r - rb) * (r - rb));
    const R ep = rexp(-alpha * (r + rb) * (r + rb));
    const R ix = rinv(x);
    // d/dr with dx/dr = 2 alpha rb, dem/dr = -2 alpha (r - rb) em, dep/dr = -2 alpha (r + rb) ep
    const R dx = (R)2 * alpha * rb;
    const R dem = -(R)2 * alpha * (r - rb) * em, dep = -(R)2 * alpha * (r + rb) * ep;
    const R dix = -dx * ix * ix;
    R v0 = (R)0.5 * (em - ep) * ix;
    R d0 = (R)0.5 * (dem - dep) * ix + (R)0.5 * (em - ep) * dix;
    out[0] = scale * v0;
    if (dout) dout[0] = d0;
    if (L < 2) return;
    R v1 = (R)0.5 * (em + ep) * ix - (R)0.5 * (em - ep) * ix * ix;
    R d1 = (R)0.5 * (dem + dep) * ix + (R)0.5 * (em + ep) * dix - (R)0.5 * (dem - dep) * ix * ix -
           (R)0.5 * (em - ep) * (R)2 * ix * dix;
    out[stride] = scale * v1;
    if (dout) dout[stride] = d1;
    for (int l = 2; l < L; ++l) {
        const R v2 = v0 - (R)(2 * l - 1) * v1 * ix;
        out[l * stride] = scale * v2;
        if (dout) {
            const R d2 = d0 - (R)(2 * l - 1) * (d1 * ix + v1 * dix);
            dout[l * stride] = d2;
            d0 = d1;
            d1 = d2;
        }
        v0 = v1;
        v1 = v2;
    }
}

__device__ __forceinline__ int species_channel(const SoapConst& sc, int z) {
    for (int s = 0; s < sc.n_species; ++s)
        if (sc.species_Z[s] == z || sc.species_Z[s] == 0) return s;
    return -1;
}

// Row pr of the power spectrum -> (ia, jb <= ia), pr = ia (ia + 1) / 2 + jb.  The FP32
// square root is a first guess (exact for pr < 2^21); the loops make the result exact.
__device__ __forceinline__ void decode_pair(int pr, int& ia, int& jb) {
    int a = (int)((sqrtf((float)(8 * pr + 1)) - 1.0f) * 0.5f);
    while ((a + 1) * (a + 2) / 2 <= pr) ++a;
    while (a * (a + 1) / 2 > pr) --a;
    ia = a;
    jb = pr - a * (a + 1) / 2;
}

__device__ __forceinline__ int l_of_lm(int lm) {
    int l = (int)sqrtf((float)lm);
    while ((l + 1) * (l + 1) <= lm) ++l;
    while (l * l > lm) --l;
    return l;
}

constexpr int FWD_THREADS = 256;
constexpr int TC = 32;   // neighbours staged per chunk in the forward kernel
constexpr int TCB = 16;  // ... and in the backward kernel (dual Ylm staging is 4x larger)
static_assert(TC == 32 && TCB == 16, "the neighbour-function phases map lanes to staged neighbours");

// Neighbour data of one chunk, loaded into registers one chunk ahead of its staging so
// that the dependent loads (list -> atomic number) overlap the previous chunk's work:
// warp 0 holds |r| and Z of neighbour base + lane (species lists), the next threads
// hold the displacement of neighbour base + (tid - 32) (staging).
struct ChunkFetch {
    double r = 0.0;
    int z = 0;
    double4 d = {0.0, 0.0, 0.0, 0.0};
    template <int TCX>
    __device__ __forceinline__ void load(int b, int p1, const int* __restrict__ Z, const int* __restrict__ nj,
                                         const double4* __restrict__ nd) {
        const int c = min(TCX, p1 - b), tid = threadIdx.x;
        if (tid < 32) {
            if (tid < c) {
                r = nd[b + tid].w;
                z = Z[nj[b + tid]];
            }
        } else if (tid - 32 < c) {
            d = nd[b + tid - 32];
        }
    }
};

// Per-chunk set-up by warp 0: species channel of each staged neighbour and, per
// species, the list of staged neighbours in staging order (deterministic).
template <int TCX>
__device__ __forceinline__ void build_species_lists(const SoapConst& sc, int cnt, const ChunkFetch& f, int* spc,
                                                    int* lst, int* lcnt) {
    const int lane = threadIdx.x & 31;
    int s = -1;
    if (lane < cnt) s = (f.r < sc.rc) ? species_channel(sc, f.z) : -1;
    if (lane < TCX) spc[lane] = s;
    const unsigned lt = (1u << lane) - 1u;
    for (int k = 0; k < sc.n_species; ++k) {
        unsigned m = __ballot_sync(0xffffffffu, s == k);
        if (s == k) lst[k * TCX + __popc(m & lt)] = lane;
        if (lane == 0) lcnt[k] = __popc(m);
    }
}

// Stage neighbour t of the chunk: unit vector, 1/r and r in R (one conversion from the
// FP64 list per neighbour), cutoff function and its derivative.
template <class R>
__device__ __forceinline__ void stage_neighbour(const SoapConst& sc, const double4& d, R* dsm, R* fcs, R* dfcs) {
    const R r = (R)d.w, ir = rinv(r);
    dsm[0] = (R)d.x * ir;
    dsm[1] = (R)d.y * ir;
    dsm[2] = (R)d.z * ir;
    dsm[3] = ir;
    dsm[4] = r;
    R f, df;
    cutoff_fn<R>(r, (R)sc.rc, (R)sc.w, f, df);
    *fcs = f;
    if (dfcs) *dfcs = df;
}
constexpr int DS = 5;  // staged values per neighbour: ux, uy, uz, 1/r, r

// sum_e h[e] * x[e] over NMP entries (NMP a multiple of 4), two right-hand sides.  The
// FP32 form keeps even and odd entries in the two halves of packed FP32x2 FMAs.
__device__ __forceinline__ void dot2(const float* __restrict__ h, const float* __restrict__ x, const float* __restrict__ y,
                                     int NMP, float& u, float& w) {
    const float4* h4 = reinterpret_cast<const float4*>(h);
    const float4* x4 = reinterpret_cast<const float4*>(x);
    const float4* y4 = reinterpret_cast<const float4*>(y);
    float2 uu = make_float2(0.f, 0.f), ww = make_float2(0.f, 0.f);
#pragma unroll
    for (int a = 0; a < MAX_NMAX / 4; ++a)
        if (a < NMP / 4) {
            const float4 hh = h4[a], xx = x4[a], yy = y4[a];
            const float2 h0 = make_float2(hh.x, hh.y), h1 = make_float2(hh.z, hh.w);
            uu = __ffma2_rn(h0, make_float2(xx.x, xx.y), uu);
            ww = __ffma2_rn(h0, make_float2(yy.x, yy.y), ww);
            uu = __ffma2_rn(h1, make_float2(xx.z, xx.w), uu);
            ww = __ffma2_rn(h1, make_float2(yy.z, yy.w), ww);
        }
    u += uu.x + uu.y;
    w += ww.x + ww.y;
}
__device__ __forceinline__ void dot2(const double* __restrict__ h, const double* __restrict__ x,
                                     const double* __restrict__ y, int NMP, double& u, double& w) {
    for (int a = 0; a < NMP; ++a) {
        u += h[a] * x[a];
        w += h[a] * y[a];
    }
}

// d0 = sum_b h[b * NNP] c[b * L2], d1 = sum_b h[b * NNP + 1] c[b * L2] (h 8-byte aligned)
__device__ __forceinline__ void hrow2(const float* __restrict__ h, const float* __restrict__ c, int NN, int NNP, int L2,
                                      float& d0, float& d1) {
    float2 acc = make_float2(0.f, 0.f);
#pragma unroll 4
    for (int b = 0; b < NN; ++b) {
        const float2 hv = *reinterpret_cast<const float2*>(h + b * NNP);
        const float cv = c[b * L2];
        acc = __ffma2_rn(hv, make_float2(cv, cv), acc);
    }
    d0 = acc.x;
    d1 = acc.y;
}
__device__ __forceinline__ void hrow2(const double* __restrict__ h, const double* __restrict__ c, int NN, int NNP,
                                      int L2, double& d0, double& d1) {
    double x = 0, y = 0;
    for (int b = 0; b < NN; ++b) {
        const double cv = c[b * L2];
        x += h[b * NNP] * cv;
        y += h[b * NNP + 1] * cv;
    }
    d0 = x;
    d1 = y;
}

template <class R>
__device__ __forceinline__ R warp_sum(R v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sums of four values over the warp, returned in every lane: a transposing butterfly
// (each of the first two exchanges sends half of the lane's partial sums), then the
// four totals are gathered from lanes 0, 8, 16 and 24.
template <class R>
__device__ __forceinline__ void warp_sum4(R& a, R& b, R& c, R& d) {
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31;
    const bool h16 = lane & 16, h8 = lane & 8;
    R k0 = h16 ? c : a, k1 = h16 ? d : b;
    k0 += __shfl_xor_sync(full, h16 ? a : c, 16);
    k1 += __shfl_xor_sync(full, h16 ? b : d, 16);
    R k = h8 ? k1 : k0;
    k += __shfl_xor_sync(full, h8 ? k0 : k1, 8);
    k += __shfl_xor_sync(full, k, 4);
    k += __shfl_xor_sync(full, k, 2);
    k += __shfl_xor_sync(full, k, 1);
    a = __shfl_sync(full, k, 0);
    b = __shfl_sync(full, k, 8);
    c = __shfl_sync(full, k, 16);
    d = __shfl_sync(full, k, 24);
}

// Global -> shared copy of n values by the block, U loads in flight per thread.
template <int U, class R>
__device__ __forceinline__ void copy_to_smem(const R* __restrict__ g, R* s, int n) {
    const int bd = blockDim.x;
    for (int k0 = threadIdx.x; k0 < n; k0 += U * bd) {
        R v[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * bd;
            v[u] = k < n ? g[k] : (R)0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const int k = k0 + u * bd;
            if (k < n) s[k] = v[u];
        }
    }
}

// A flattened loop index k = i * B + j walked with a fixed stride S: (i, j) advance
// without an integer division per step (S / B and S % B are formed once).
struct Walk2 {
    int i, j, si, sj, B;
    __device__ __forceinline__ Walk2(int k, int S, int B_) : B(B_) {
        i = k / B;
        j = k - i * B;
        si = S / B;
        sj = S - si * B;
    }
    __device__ __forceinline__ void next() {
        i += si;
        j += sj;
        if (j >= B) {
            j -= B;
            ++i;
        }
    }
};

__device__ __forceinline__ void load4(const float* p, float& a, float& b, float& c, float& d) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    a = v.x; b = v.y; c = v.z; d = v.w;
}
__device__ __forceinline__ void load4(const double* p, double& a, double& b, double& c, double& d) {
    const double2 u = reinterpret_cast<const double2*>(p)[0], v = reinterpret_cast<const double2*>(p)[1];
    a = u.x; b = u.y; c = v.x; d = v.y;
}

// Accumulator items a forward thread keeps in registers: FQ_SMALL for bases of up to
// FQ_SMALL * 256 items (s, lm, 4 radial functions), FQ_LARGE beyond.
constexpr int FQ_SMALL = 2, FQ_LARGE = 8;

// Size (elements) of the forward kernel's shared region: staging, ct or power spectrum.
__host__ __device__ __forceinline__ int fwd_region(const SoapConst& sc) {
    const int L = sc.l_max + 1, L2 = L * L, NMP = nmp_of(sc.n_max);
    int r = TC * L2 + TC * L * NMP + TC + TC * DS;
    r = r > sc.n_species * L2 * NMP ? r : sc.n_species * L2 * NMP;
    r = r > sc.n_pairs * L ? r : sc.n_pairs * L;
    return (r + 3) & ~3;
}

// Forward: one block per centre.  Densities are accumulated in the collocation basis
// ct[s][lm][a] = sum_j fc rho_l(r_j, r_a) Y_lm(r^_j): each thread owns up to FQ items
// (s, lm, 4 consecutive a) in registers for the whole neighbour loop.  The
// orthonormalising transform c[s][n][lm] = sum_a T_an ct[s][lm][a] is applied once per
// centre by one thread per (s, lm).  In the mixed path everything is FP32 except the
// norm reduction (per-thread FP32 partial sums combined in FP64) and 1/|p|.
template <class R, int FQ>
__global__ void __launch_bounds__(FWD_THREADS) k_soap_forward(SoapConst sc, const R* __restrict__ tab, int nc,
                                                               const int* __restrict__ centres, const int* __restrict__ Z,
                                                               const int* __restrict__ off, const int* __restrict__ nj,
                                                               const double4* __restrict__ nd, R* __restrict__ c_out,
                                                               R* __restrict__ q_out, void* __restrict__ qr_out, int qr_half,
                                                               double* __restrict__ pnorm) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ci = blockIdx.x;
    if (ci >= nc) return;
    const int atom = centres[ci];
    const int L = sc.l_max + 1, L2 = L * L, nm = sc.n_max, NMP = nmp_of(nm), NS = sc.n_species;
    const SoapTab tb = soap_tab(nm, L);
    // [K][cs][region]: the region holds the neighbour staging during the loop, then the
    // accumulators ct for the transform, then the power spectrum (ct is dead by then)
    R* K = reinterpret_cast<R*>(smem_raw);           // tb.size
    R* cs = K + tb.size;                              // NS * nm * L2
    R* Ysm = cs + ((NS * nm * L2 + 3) & ~3);          // TC * L2
    R* Ism = Ysm + TC * L2;                           // TC * L * NMP
    R* fcs = Ism + TC * L * NMP;                      // TC
    R* dsm = fcs + TC;                                // TC * DS
    R* ct = Ysm;                                      // NS * L2 * NMP, after the loop
    const int region = fwd_region(sc);
    int* spc = reinterpret_cast<int*>(Ysm + region);  // TC
    int* lst = spc + TC;                              // NS * TC
    int* lcnt = lst + NS * TC;                        // NS
    unsigned char* lofm = reinterpret_cast<unsigned char*>(lcnt + NS);  // L2
    const int tid = threadIdx.x, bd = blockDim.x;
    copy_to_smem<4>(tab, K, tb.size);
    for (int k = tid; k < L2; k += bd) lofm[k] = (unsigned char)l_of_lm(k);
    const int NA4 = NMP / 4, items = NS * L2 * NA4;  // NA4 also sizes the transform's vector loads

    R acc[FQ][4];
    int own_s[FQ], own_lm[FQ], own_a4[FQ];
#pragma unroll
    for (int q = 0; q < FQ; ++q) {
        const int k = tid + q * bd;
        own_s[q] = -1;
        own_lm[q] = own_a4[q] = 0;
        if (k < items) {
            own_s[q] = k / (L2 * NA4);
            const int rem = k - own_s[q] * L2 * NA4;
            own_lm[q] = rem / NA4;
            own_a4[q] = rem - own_lm[q] * NA4;
        }
        acc[q][0] = acc[q][1] = acc[q][2] = acc[q][3] = 0;
    }
    const R alpha = (R)sc.alpha;
    const int NPAD = NMP - nm;  // basis columns n_max..NMP-1 of the staged radial rows stay zero
    for (int k = tid; k < TC * L * NPAD; k += bd) {
        const int row = k / NPAD;
        Ism[row * NMP + nm + (k - row * NPAD)] = 0;
    }
    const int p0 = off[atom], p1 = off[atom + 1];
    for (int base = p0; base < p1; base += TC) {
        const int cnt = min(TC, p1 - base);
        __syncthreads();
        {
            ChunkFetch nf;  // loaded where it is staged: registers are this kernel's occupancy limit
            nf.load<TC>(base, p1, Z, nj, nd);
            if (tid < 32) build_species_lists<TC>(sc, cnt, nf, spc, lst, lcnt);
            else if (tid - 32 < cnt) {
                const int t = tid - 32;
                stage_neighbour<R>(sc, nf.d, dsm + DS * t, fcs + t, (R*)nullptr);
            }
        }
        __syncthreads();
        // Ylm columns and radial rows of the staged neighbours: lane = neighbour, each warp
        // runs its task list (warp-uniform branches, no per-task index decoding)
        {
            const int t = tid & 31, wid = tid >> 5;
            const bool act = t < cnt && spc[t] >= 0;
            R ux = 0, uy = 0, uz = 1, r = 1, fc = 0;
            if (act) {
                const R* u = dsm + DS * t;
                ux = u[0]; uy = u[1]; uz = u[2]; r = u[4]; fc = fcs[t];
            }
#pragma unroll 1
            for (int j = 0; j < 8; ++j) {
                const int task = sc.fsched[wid][j];
                if (task == 0xff) break;
                if (!act) continue;
                if (task < nm) radial_collocation<R>(r, K[tb.rb + task], alpha, L, fc, Ism + t * L * NMP + task, (R*)nullptr, NMP);
                else ylm_column<R>(task - nm, L, ux, uy, uz, K, tb, Ysm + t * L2);
            }
        }
        __syncthreads();
        // acc[s][lm][a..a+3] += sum_{t in species s} Y[t][lm] I[t][l][a..a+3]
#pragma unroll
        for (int q = 0; q < FQ; ++q) {
            const int s = own_s[q];
            if (s < 0) continue;
            const int lm = own_lm[q], l = lofm[lm], a4 = own_a4[q];
            const int nt = lcnt[s];
            const int* ls = lst + s * TC;
            for (int qq = 0; qq < nt; ++qq) {
                const int t = ls[qq];
                const R y = Ysm[t * L2 + lm];
                R i0, i1, i2, i3;
                load4(Ism + (t * L + l) * NMP + 4 * a4, i0, i1, i2, i3);
                acc[q][0] += y * i0; acc[q][1] += y * i1; acc[q][2] += y * i2; acc[q][3] += y * i3;
            }
        }
    }
    __syncthreads();  // the staging area becomes ct
#pragma unroll
    for (int q = 0; q < FQ; ++q) {
        if (own_s[q] < 0) continue;
        R* o = ct + (own_s[q] * L2 + own_lm[q]) * NMP + 4 * own_a4[q];
        o[0] = acc[q][0]; o[1] = acc[q][1]; o[2] = acc[q][2]; o[3] = acc[q][3];
    }
    __syncthreads();
    // c[s][n][lm] = sum_a T_an ct[s][lm][a]  (+ central atom at l = 0): one thread per (s, lm)
    const int zc = Z[atom];
    for (int k = tid; k < NS * L2; k += bd) {
        const int s = k / L2, lm = k - s * L2;
        const R* v = ct + (s * L2 + lm) * NMP;
        R va[MAX_NMAX];
#pragma unroll
        for (int a4 = 0; a4 < MAX_NMAX / 4; ++a4)
            if (a4 < NA4) load4(v + 4 * a4, va[4 * a4], va[4 * a4 + 1], va[4 * a4 + 2], va[4 * a4 + 3]);
        const bool centre = lm == 0 && (sc.centre_all || sc.species_Z[s] == zc || sc.species_Z[s] == 0);
        for (int n = 0; n < nm; ++n) {
            const R* tr = K + tb.Tt + n * NMP;
            R x = 0;
#pragma unroll
            for (int a4 = 0; a4 < MAX_NMAX / 4; ++a4)
                if (a4 < NA4) {
                    R t0, t1, t2, t3;
                    load4(tr + 4 * a4, t0, t1, t2, t3);
                    x += t0 * va[4 * a4] + t1 * va[4 * a4 + 1] + t2 * va[4 * a4 + 2] + t3 * va[4 * a4 + 3];
                }
            if (centre) x += K[tb.cr + n];
            cs[(s * nm + n) * L2 + lm] = x;
        }
    }
    __syncthreads();
    R* cg = c_out + (size_t)ci * sc.ncomp;
    for (int k = tid; k < sc.ncomp; k += bd) cg[k] = cs[k];
    // power spectrum: one item per (l, 2x2 block of channel rows (ia, jb), ia >= jb), so
    // that each pair of loaded coefficients feeds two products
    R* ps = Ysm;
    R ssr = 0;
    {
        const int NR = NS * nm, NB = (NR + 1) / 2, nblk = NB * (NB + 1) / 2;
        if (tid < nblk * L) {
            Walk2 w(tid, bd, nblk);
            for (; w.i < L; w.next()) {
                const int l = w.i;
                int bi = (int)((sqrtf((float)(8 * w.j + 1)) - 1.0f) * 0.5f);
                while ((bi + 1) * (bi + 2) / 2 <= w.j) ++bi;
                while (bi * (bi + 1) / 2 > w.j) --bi;
                const int bj = w.j - bi * (bi + 1) / 2;
                const int i0 = 2 * bi, j0 = 2 * bj;
                const bool i1ok = i0 + 1 < NR, j1ok = j0 + 1 < NR;
                const R* a0 = cs + i0 * L2 + l * l;
                const R* a1 = cs + (i1ok ? i0 + 1 : i0) * L2 + l * l;
                const R* b0 = cs + j0 * L2 + l * l;
                const R* b1 = cs + (j1ok ? j0 + 1 : j0) * L2 + l * l;
                R v00 = 0, v01 = 0, v10 = 0, v11 = 0;
                for (int m = 0; m < 2 * l + 1; ++m) {
                    const R x0 = a0[m], x1 = a1[m], y0 = b0[m], y1 = b1[m];
                    v00 += x0 * y0;
                    v01 += x0 * y1;
                    v10 += x1 * y0;
                    v11 += x1 * y1;
                }
                const R lf = K[tb.lf + l], r2 = (R)1.41421356237309504880;
                auto put = [&](int ia, int jb, R v) {
                    v *= (ia != jb ? r2 : (R)1) * lf;
                    ps[(ia * (ia + 1) / 2 + jb) * L + l] = v;
                    ssr += v * v;
                };
                put(i0, j0, v00);
                if (j1ok && bi != bj) put(i0, j0 + 1, v01);
                if (i1ok) put(i0 + 1, j0, v10);
                if (i1ok && j1ok) put(i0 + 1, j0 + 1, v11);
            }
        }
    }
    // FP32 partial sums per warp, combined in FP64
    __shared__ double s_wsum[FWD_THREADS / 32];
    __shared__ R s_inv;
    ssr = warp_sum(ssr);
    if ((tid & 31) == 0) s_wsum[tid >> 5] = (double)ssr;
    __syncthreads();
    if (tid == 0) {
        double tot = 0;
        for (int w = 0; w < FWD_THREADS / 32; ++w) tot += s_wsum[w];
        const double nrm = sqrt(tot);
        pnorm[ci] = nrm;
        s_inv = sc.normalise ? (R)(1.0 / nrm) : (R)1;
    }
    __syncthreads();
    const R inv = s_inv;
    const int np = sc.n_pairs * L;
    R* qg = q_out + (size_t)ci * sc.dpad;
    // the first GEMM's operand next to q: TF32-rounded FP32, or FP16 for the FP16 GEMM
    float* qrg = qr_out && !qr_half ? static_cast<float*>(qr_out) + (size_t)ci * sc.dpad : nullptr;
    __half* qhg = qr_out && qr_half ? static_cast<__half*>(qr_out) + (size_t)ci * sc.dpad : nullptr;
    for (int k = tid; k < sc.dpad; k += bd) {
        R v;
        if (k < np) v = ps[k] * inv;
        else if (k == np) v = (R)sc.sigma0;
        else v = 0;
        qg[k] = v;
        if (qrg) __stcs(qrg + k, round_tf32((float)v));
        if (qhg) qhg[k] = __float2half_rn((float)v);
    }
}

constexpr int BWD_THREADS = 256;
static_assert(FWD_THREADS == 256 && BWD_THREADS == 256, "8 warps: the rows of the task schedules");
constexpr int BWD_WARPS = BWD_THREADS / 32;

// Shared-memory plan of the backward kernel (elements of R): constant block, h, then a
// region used first for (c, dE/dc, dE/dp) and then for the neighbour staging.
struct BwdPlan {
    int hs, U, pre, stage, ints_at;
};
__host__ __device__ __forceinline__ BwdPlan bwd_plan(const SoapConst& sc) {
    const int L = sc.l_max + 1, L2 = L * L, NMP = nmp_of(sc.n_max), NS = sc.n_species;
    BwdPlan p;
    p.hs = soap_tab(sc.n_max, L).size;
    p.U = p.hs + ((NS * L2 * NMP + 7) & ~7);
    const int NN = NS * sc.n_max, NNP = (NN + 1) & ~1;
    p.pre = 2 * ((sc.ncomp + 3) & ~3) + L * NN * NNP;  // c, dE/dc, symmetric dE/dp matrices
    p.stage = 4 * TCB * L2 + 2 * TCB * L * NMP + (2 + DS) * TCB;
    p.ints_at = p.U + (((p.pre > p.stage ? p.pre : p.stage) + 7) & ~7);
    return p;
}

// Backward: one block per centre.
//   dE/dp (normalisation Jacobian: FP64 scalars q.G and 1/|p|) -> H_l[a][b]
//   dE/dc[a][lm] = sum_b H_l[a][b] c[b][lm]
//   h[s][lm][a'] = sum_n T_a'n dE/dc[s][n][lm]        (back to the collocation basis)
//   per pair t of species s:  u_lm = sum_a h[s][lm][a] rho_al(r),  w_lm = sum_a h[s][lm][a] drho_al/dr
//   f_t = sum_lm [(fc w_lm + fc' u_lm) Y_lm r^ + fc u_lm grad Y_lm]
template <class R>
__global__ void __launch_bounds__(BWD_THREADS) k_soap_backward(SoapConst sc, const R* __restrict__ tab, int nc,
                                                                const int* __restrict__ centres, const int* __restrict__ Z,
                                                                const int* __restrict__ off, const int* __restrict__ nj,
                                                                const double4* __restrict__ nd, const R* __restrict__ c_in,
                                                                const R* __restrict__ q_in, const double* __restrict__ pnorm,
                                                                const R* __restrict__ G, double* __restrict__ fpair) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    const int ci = blockIdx.x;
    if (ci >= nc) return;
    const int atom = centres[ci];
    const int L = sc.l_max + 1, L2 = L * L, nm = sc.n_max, NMP = nmp_of(nm), NS = sc.n_species, NN = NS * nm;
    const int np = sc.n_pairs * L;
    const SoapTab tb = soap_tab(nm, L);
    const BwdPlan pl = bwd_plan(sc);
    R* K = reinterpret_cast<R*>(smem_raw);
    R* hs = K + pl.hs;                                  // NS * L2 * NMP
    R* U = K + pl.U;
    // pre-phase view of U
    const int NNP = (NN + 1) & ~1;                      // row length of the dE/dp matrices (even)
    R* cs = U;                                          // ncomp
    R* dc = cs + ((sc.ncomp + 3) & ~3);                 // ncomp
    R* Hf = dc + ((sc.ncomp + 3) & ~3);                 // L * NN * NNP: H_l[b][a] = dE/dp(pair(a, b), l)
    // staging view of U
    Dual<R>* Yd = reinterpret_cast<Dual<R>*>(U);        // TCB * L2
    R* Ism = U + 4 * TCB * L2;                          // TCB * L * NMP
    R* dIsm = Ism + TCB * L * NMP;                      // TCB * L * NMP
    R* fcs = dIsm + TCB * L * NMP;                      // TCB
    R* dfcs = fcs + TCB;                                // TCB
    R* dsm = dfcs + TCB;                                // TCB * DS
    int* spc = reinterpret_cast<int*>(K + pl.ints_at);  // TCB
    int* lst = spc + TCB;                               // NS * TCB
    int* lcnt = lst + NS * TCB;                         // NS
    unsigned char* lofm = reinterpret_cast<unsigned char*>(lcnt + NS);  // L2
    unsigned short* ptab = reinterpret_cast<unsigned short*>(lofm + ((L2 + 1) & ~1));  // n_pairs: ia << 8 | jb
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5, bd = blockDim.x;
    const int p0 = off[atom], p1 = off[atom + 1];
    ChunkFetch nf;
    if (p0 < p1) nf.load<TCB>(p0, p1, Z, nj, nd);
    // q.G, the entries of this thread's first QU strides kept in registers for dE/dp
    constexpr int QU = 8;
    const R* qg = q_in + (size_t)ci * sc.dpad;
    const R* gg = G + (size_t)ci * sc.dpad;
    R qv[QU], gv[QU];
#pragma unroll
    for (int u = 0; u < QU; ++u) {
        const int k = tid + u * bd;
        qv[u] = k < np ? qg[k] : (R)0;
        gv[u] = k < np ? gg[k] : (R)0;
    }
    copy_to_smem<4>(tab, K, tb.size);
    copy_to_smem<8>(c_in + (size_t)ci * sc.ncomp, cs, sc.ncomp);
    for (int k = tid; k < L2; k += bd) lofm[k] = (unsigned char)l_of_lm(k);
    for (int pr = tid; pr < sc.n_pairs; pr += bd) {
        int ia, jb;
        decode_pair(pr, ia, jb);
        ptab[pr] = (unsigned short)(ia << 8 | jb);
    }
    if (NNP > NN)
        for (int k = tid; k < L * NN; k += bd) Hf[k * NNP + NN] = 0;
    R part = 0;
#pragma unroll
    for (int u = 0; u < QU; ++u) part += qv[u] * gv[u];
    for (int k = tid + QU * bd; k < np; k += bd) part += qg[k] * gg[k];
    __shared__ double s_wsum[BWD_WARPS];
    __shared__ R s_sc[2];
    __shared__ R s_f[3 * TCB];  // per-pair forces of the last chunk, flushed during the next staging
    part = warp_sum(part);
    if (lane == 0) s_wsum[wid] = (double)part;
    __syncthreads();
    if (tid == 0) {
        double tot = 0;
        for (int w = 0; w < BWD_WARPS; ++w) tot += s_wsum[w];
        s_sc[0] = (R)tot;
        s_sc[1] = (R)(1.0 / pnorm[ci]);
    }
    __syncthreads();
    const R sq = s_sc[0], inv = s_sc[1];
    // dE/dp[pair * L + l] into the symmetric matrices H_l (both triangles)
    {
        Walk2 w(tid, bd, L);  // (pair, l) of k = tid + u * bd
        auto put = [&](int pr, int l, R q, R g) {
            const int ia = ptab[pr] >> 8, jb = ptab[pr] & 255;
            const R f0 = ia != jb ? (R)1.41421356237309504880 : (R)2;
            const R v = (sc.normalise ? (g - q * sq) * inv : g) * f0 * K[tb.lf + l];
            R* H = Hf + l * NN * NNP;
            H[ia * NNP + jb] = v;
            H[jb * NNP + ia] = v;
        };
#pragma unroll
        for (int u = 0; u < QU; ++u) {
            if (tid + u * bd < np) put(w.i, w.j, qv[u], gv[u]);
            w.next();
        }
        for (int k = tid + QU * bd; k < np; k += bd, w.next()) put(w.i, w.j, qg[k], gg[k]);
    }
    __syncthreads();
    // dE/dc[a][lm] = sum_b H_l[b][a] c[b][lm], rows a and a + 1 per thread; the row pair
    // is fastest, so a warp reads few distinct c and consecutive H entries
    {
        Walk2 w(tid, bd, NNP / 2);
        for (; w.i < L2; w.next()) {
            const int lm = w.i, a = 2 * w.j;
            R d0, d1;
            hrow2(Hf + lofm[lm] * NN * NNP + a, cs + lm, NN, NNP, L2, d0, d1);
            dc[a * L2 + lm] = d0;
            if (a + 1 < NN) dc[(a + 1) * L2 + lm] = d1;
        }
    }
    __syncthreads();
    // h[s][lm][a] = sum_n T_an dE/dc[s][n][lm]: one thread per (s, lm)
    const int NN4 = NMP / 4;
    for (int k = tid; k < NS * L2; k += bd) {
        const int s = k / L2, lm = k - s * L2;
        R vn[MAX_NMAX];
#pragma unroll
        for (int n = 0; n < MAX_NMAX; ++n) vn[n] = n < nm ? dc[(s * nm + n) * L2 + lm] : (R)0;
        R* o = hs + (s * L2 + lm) * NMP;
        for (int a = 0; a < NMP; ++a) {  // Tp rows beyond n_max are zero
            const R* tr = K + tb.Tp + a * NMP;
            R x = 0;
#pragma unroll
            for (int n4 = 0; n4 < MAX_NMAX / 4; ++n4)
                if (n4 < NN4) {
                    R t0, t1, t2, t3;
                    load4(tr + 4 * n4, t0, t1, t2, t3);
                    x += t0 * vn[4 * n4] + t1 * vn[4 * n4 + 1] + t2 * vn[4 * n4 + 2] + t3 * vn[4 * n4 + 3];
                }
            o[a] = x;
        }
    }
    const R alpha = (R)sc.alpha;
    int prev = p0, prev_cnt = 0;
    for (int base = p0; base < p1; base += TCB) {
        const int cnt = min(TCB, p1 - base);
        __syncthreads();
        if (tid < 32) build_species_lists<TCB>(sc, cnt, nf, spc, lst, lcnt);
        else if (tid - 32 < cnt) {
            const int t = tid - 32;
            stage_neighbour<R>(sc, nf.d, dsm + DS * t, fcs + t, dfcs + t);
        } else if (tid >= 64 && tid - 64 < 3 * prev_cnt) {
            fpair[3 * (size_t)prev + (tid - 64)] += (double)s_f[tid - 64];
        }
        if (base == p0 && tid >= 64) {
            // basis columns n_max..NMP-1 of the staged radial rows stay zero (the staging
            // area held the pre-phase buffers until now)
            const int NPAD = NMP - nm;
            for (int k = tid - 64; k < TCB * L * NPAD; k += bd - 64) {
                const int row = k / NPAD, col = nm + (k - row * NPAD);
                Ism[row * NMP + col] = 0;
                dIsm[row * NMP + col] = 0;
            }
        }
        prev = base;
        prev_cnt = cnt;
        __syncthreads();
        if (base + TCB < p1) nf.load<TCB>(base + TCB, p1, Z, nj, nd);
        // one task list: Ylm columns (m descending, neighbour fastest, so a warp's lanes
        // share m and the recurrences run equally long), then the radial rows (t, a) with
        // their r-derivatives
        const int nY = cnt * L, nT = nY + cnt * nm;
        for (int k = tid; k < nT; k += bd) {
            if (k < nY) {
                const int mi = k / cnt, t = k - mi * cnt;
                if (spc[t] < 0) continue;
                const R* u = dsm + DS * t;
                ylm_column_cart<R>(L - 1 - mi, L, u[0], u[1], u[2], K, tb, Yd + t * L2);
            } else {
                const int k2 = k - nY, t = k2 / nm, a = k2 - t * nm;
                if (spc[t] < 0) continue;
                radial_collocation<R>(dsm[DS * t + 4], K[tb.rb + a], alpha, L, (R)1, Ism + t * L * NMP + a,
                                      dIsm + t * L * NMP + a, NMP);
            }
        }
        __syncthreads();
        for (int t = wid; t < cnt; t += BWD_WARPS) {
            const int s = spc[t];
            if (s < 0) {  // warp-uniform
                if (lane < 3) s_f[3 * t + lane] = 0;
                continue;
            }
            const R* u = dsm + DS * t;
            const R ux = u[0], uy = u[1], uz = u[2], ir = u[3];
            const R f = fcs[t], df = dfcs[t];
            // radial part sum_lm (f w + f' u) Y and angular part sum_lm f u dY/du (unprojected)
            R ar = 0, gx = 0, gy = 0, gz = 0;
            for (int lm = lane; lm < L2; lm += 32) {
                const int l = lofm[lm];
                R uu = 0, ww = 0;
                dot2(hs + (s * L2 + lm) * NMP, Ism + (t * L + l) * NMP, dIsm + (t * L + l) * NMP, NMP, uu, ww);
                const Dual<R> y = Yd[t * L2 + lm];
                const R ang = f * uu;
                ar += (f * ww + df * uu) * y.v;
                gx += ang * y.x;
                gy += ang * y.y;
                gz += ang * y.z;
            }
            warp_sum4(ar, gx, gy, gz);
            if (lane == 0) {
                // f = ar u + (I - u u^T) g / r
                const R gu = gx * ux + gy * uy + gz * uz;
                const R fx = ar * ux + (gx - gu * ux) * ir;
                const R fy = ar * uy + (gy - gu * uy) * ir;
                const R fz = ar * uz + (gz - gu * uz) * ir;
                s_f[3 * t] = fx;
                s_f[3 * t + 1] = fy;
                s_f[3 * t + 2] = fz;
            }
        }
    }
    __syncthreads();
    if (tid < 3 * prev_cnt) fpair[3 * (size_t)prev + tid] += (double)s_f[tid];
}

// FP32 backward in two kernels.  k_soap_bwd_h: one block per centre forms
//   h[s][lm][a] = sum_n T_an dE/dc[s][n][lm],  dE/dc[a][lm] = sum_b H_l[a][b] c[b][lm]
// (H_l the symmetric dE/dp matrices) as k_soap_backward does, into a global buffer.
// k_soap_bwd_pairs: one thread per pair (all pairs of all centres, so no lane idles
// at the end of a short neighbour list) walks l and m upwards with everything of the
// pair in registers (basis sizes fixed at compile time: L = l_max + 1, NMP = n_max
// padded to 4): the radial functions of all grid points a (upward recurrence
// rho_{l+1} = rho_{l-1} - (2l+1)/x rho_l) and the Legendre columns of all m (the
// recurrences of ylm_column_cart, reordered l-outer, their constants in constant
// memory).  The radial derivative needs no second recurrence: i_l'(x) = i_{l-1}(x) -
// (l+1)/x i_l(x) gives, for rb > 0,
//   d rho_l/dr = -(2 alpha r + (l+1)/r) rho_l + 2 alpha rb rho_{l-1},  rho_{-1} = (e- + e+)/2x,
// so sum_lm w_lm Y_lm = sum_l c_l sum_m u_lm Y_lm + 2 alpha sum_lm v_lm Y_lm with
// v_lm = sum_a h[lm][a] rb_a rho_{a,l-1} and c_l = -(2 alpha r + (l+1)/r).  The +m and -m
// entries of one (l, m) share their Legendre factor and the two Cartesian forms, so the
// sums over lm are taken per (l, m) from U1 = u+ cm + u- sm, V1 = v+ cm + v- sm,
// Ux = u+ cp + u- sp, Uy = u- cp - u+ sp.  A grid point at rb = 0 contributes
// exp(-alpha r^2) at l = 0 only and is added to the lm = 0 term.
constexpr int BH_THREADS = 256;
constexpr int BP_THREADS = 128;
constexpr int BP_SMEM_BYTES = 32 * 1024;  // h rows a pair-kernel block stages (4 centres at the headline basis)
constexpr int BH_MAXNN = 24;  // species x n_max of the register-blocked dE/dc rows
constexpr int MAX_L2 = (MAX_LMAX + 1) * (MAX_LMAX + 1);
__constant__ float c_lra[MAX_L2], c_lrbb[MAX_L2], c_lyn[MAX_L2];  // by l*l + m, as in the SoapTab

__host__ __device__ __forceinline__ int bh_nnp(const SoapConst& sc) { return (sc.n_species * sc.n_max + 3) & ~3; }
__host__ __device__ __forceinline__ size_t bh_floats(const SoapConst& sc) {
    const int L = sc.l_max + 1, c4 = (sc.ncomp + 3) & ~3, p4 = (sc.n_pairs * L + 3) & ~3;
    return (size_t)soap_tab(sc.n_max, L).size + 2 * (size_t)c4 + (size_t)L * sc.n_species * sc.n_max * bh_nnp(sc) +
           2 * (size_t)p4;
}

// Global -> shared copy of n floats by the block with cp.async (no registers held, every
// copy of the block in flight at once): 16-byte copies where both addresses and n allow,
// else 4-byte ones.  Completed by cp_async_wait() and a barrier.
__device__ __forceinline__ void cp_async_floats(float* s, const float* __restrict__ g, int n) {
    const bool v16 = (((uintptr_t)g | (uintptr_t)s) & 15) == 0 && (n & 3) == 0;
    if (v16) {
        for (int k = 4 * (int)threadIdx.x; k < n; k += 4 * (int)blockDim.x)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"((unsigned)__cvta_generic_to_shared(s + k)),
                         "l"(g + k) : "memory");
    } else {
        for (int k = threadIdx.x; k < n; k += blockDim.x)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((unsigned)__cvta_generic_to_shared(s + k)),
                         "l"(g + k) : "memory");
    }
}
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.commit_group;\n cp.async.wait_group 0;" ::: "memory"); }

__global__ void __launch_bounds__(BH_THREADS, 4) k_soap_bwd_h(SoapConst sc, const float* __restrict__ tab, int nc,
                                                           const float* __restrict__ c_in, const float* __restrict__ q_in,
                                                           const double* __restrict__ pnorm, const float* __restrict__ G,
                                                           float* __restrict__ hbuf) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ci = blockIdx.x;
    if (ci >= nc) return;
    const int L = sc.l_max + 1, L2 = L * L, nm = sc.n_max, NMP = nmp_of(nm), NS = sc.n_species, NN = NS * nm;
    const int NNP = bh_nnp(sc), ncomp = sc.ncomp, np = sc.n_pairs * L, c4 = (ncomp + 3) & ~3;
    const SoapTab tb = soap_tab(nm, L);
    float* K = reinterpret_cast<float*>(smem_raw);
    float* cs = K + tb.size;  // c[b][lm]
    float* dc = cs + c4;      // dE/dc[a][lm]
    float* H = dc + c4;       // H_l[a][b], rows padded to NNP (zero)
    float* qg = H + L * NN * NNP;             // q and dE/dq of this centre
    float* gg = qg + ((np + 3) & ~3);
    __shared__ double s_wsum[BH_THREADS / 32];
    __shared__ unsigned char lofm[MAX_L2];
    const int tid = threadIdx.x;
    cp_async_floats(K, tab, tb.size);
    cp_async_floats(cs, c_in + (size_t)ci * ncomp, ncomp);
    cp_async_floats(qg, q_in + (size_t)ci * sc.dpad, np);
    cp_async_floats(gg, G + (size_t)ci * sc.dpad, np);
    for (int k = tid; k < L2; k += BH_THREADS) lofm[k] = (unsigned char)l_of_lm(k);
    if (NNP > NN)
        for (int k = tid; k < L * NN; k += BH_THREADS)
            for (int b = NN; b < NNP; ++b) H[k * NNP + b] = 0.f;
    cp_async_wait();
    __syncthreads();
    float part = 0.f;
    for (int k = tid; k < np; k += BH_THREADS) part += qg[k] * gg[k];
    part = warp_sum(part);
    if ((tid & 31) == 0) s_wsum[tid >> 5] = (double)part;
    __syncthreads();
    double tot = 0;
#pragma unroll
    for (int w = 0; w < BH_THREADS / 32; ++w) tot += s_wsum[w];
    const float sq = (float)tot, inv = (float)(1.0 / pnorm[ci]);
    // dE/dp into both triangles of H_l, one power-spectrum row (ia, jb) per thread
    for (int pr = tid; pr < sc.n_pairs; pr += BH_THREADS) {
        int ia, jb;
        decode_pair(pr, ia, jb);
        const float f0 = ia != jb ? 1.41421356237309504880f : 2.f;
        for (int l = 0; l < L; ++l) {
            const int k = pr * L + l;
            const float g = gg[k];
            const float v = (sc.normalise ? (g - qg[k] * sq) * inv : g) * f0 * K[tb.lf + l];
            H[(l * NN + ia) * NNP + jb] = v;
            H[(l * NN + jb) * NNP + ia] = v;
        }
    }
    __syncthreads();
    // dE/dc: one item per (lm, 4 rows a), the column c[.][lm] in registers, rows of H_l
    // as vector loads (broadcast to the threads of one l)
    const int NA4 = (NN + 3) / 4;
    for (int it = tid; it < L2 * NA4; it += BH_THREADS) {
        const int lm = it / NA4, a0 = 4 * (it - lm * NA4), l = lofm[lm];
        float cb[BH_MAXNN];
#pragma unroll
        for (int b = 0; b < BH_MAXNN; ++b) cb[b] = b < NN ? cs[b * L2 + lm] : 0.f;
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int a = a0 + r;
            if (a >= NN) break;
            const float4* h4 = reinterpret_cast<const float4*>(H + (l * NN + a) * NNP);
            float x = 0.f;
#pragma unroll
            for (int b4 = 0; b4 < BH_MAXNN / 4; ++b4)
                if (4 * b4 < NNP) {
                    const float4 hv = h4[b4];
                    x += hv.x * cb[4 * b4] + hv.y * cb[4 * b4 + 1] + hv.z * cb[4 * b4 + 2] + hv.w * cb[4 * b4 + 3];
                }
            dc[a * L2 + lm] = x;
        }
    }
    __syncthreads();
    // h[s][lm][a] = sum_n T_an dE/dc[s n][lm] (Tp rows past n_max are zero: so is h there)
    float* ho = hbuf + (size_t)ci * NS * L2 * NMP;
    for (int it = tid; it < NS * L2; it += BH_THREADS) {
        const int s = it / L2, lm = it - s * L2;
        float vn[MAX_NMAX];
#pragma unroll
        for (int n = 0; n < MAX_NMAX; ++n) vn[n] = n < nm ? dc[(s * nm + n) * L2 + lm] : 0.f;
        float4* o = reinterpret_cast<float4*>(ho + (size_t)(s * L2 + lm) * NMP);
#pragma unroll
        for (int a4 = 0; a4 < MAX_NMAX / 4; ++a4) {
            if (4 * a4 >= NMP) break;
            float x[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) {
                const float4* tr = reinterpret_cast<const float4*>(K + tb.Tp + (4 * a4 + r) * NMP);
                float acc = 0.f;
#pragma unroll
                for (int n4 = 0; n4 < MAX_NMAX / 4; ++n4)
                    if (4 * n4 < NMP) {
                        const float4 t = tr[n4];
                        acc += t.x * vn[4 * n4] + t.y * vn[4 * n4 + 1] + t.z * vn[4 * n4 + 2] + t.w * vn[4 * n4 + 3];
                    }
                x[r] = acc;
            }
            o[a4] = make_float4(x[0], x[1], x[2], x[3]);
        }
    }
}

// The same h with the basis sizes fixed at compile time (L, NM = n_max, NS species): one
// thread per lm holds the column c[.][lm] and the accumulators dE/dc[.][lm] in registers
// and walks the packed dE/dp rows (ia, jb <= ia) unrolled, each entry a broadcast load
// (dE/dc[ia] += v c[jb], dE/dc[jb] += v c[ia]); T is applied from shared memory and the
// rows of h go straight to global memory.  No barrier after dE/dp.
template <int L, int NM, int NS>
__global__ void __launch_bounds__(((L * L + 31) / 32) * 32) k_soap_bwd_h_lm(SoapConst sc, const float* __restrict__ tab,
                                                                              int nc, const float* __restrict__ c_in,
                                                                              const float* __restrict__ q_in,
                                                                              const double* __restrict__ pnorm,
                                                                              const float* __restrict__ G,
                                                                              float* __restrict__ hbuf) {
    constexpr int L2 = L * L, NN = NS * NM, NMP = (NM + 3) & ~3, NP = NN * (NN + 1) / 2, NPL = NP * L;
    constexpr int T = ((L2 + 31) / 32) * 32, NW = T / 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ci = blockIdx.x;
    if (ci >= nc) return;
    const SoapTab tb = soap_tab(NM, L);
    float* K = reinterpret_cast<float*>(smem_raw);
    float* qs = K + tb.size;
    float* gs = qs + ((NPL + 3) & ~3);  // dE/dq, then dE/dp in place
    __shared__ double s_wsum[NW];
    const int tid = threadIdx.x, lm = tid;
    cp_async_floats(K, tab, tb.size);
    cp_async_floats(qs, q_in + (size_t)ci * sc.dpad, NPL);
    cp_async_floats(gs, G + (size_t)ci * sc.dpad, NPL);
    float creg[NN];
    const float* cg = c_in + (size_t)ci * sc.ncomp;
#pragma unroll
    for (int b = 0; b < NN; ++b) creg[b] = lm < L2 ? cg[b * L2 + lm] : 0.f;
    cp_async_wait();
    __syncthreads();
    float part = 0.f;
    for (int k = tid; k < NPL; k += T) part += qs[k] * gs[k];
    part = warp_sum(part);
    if ((tid & 31) == 0) s_wsum[tid >> 5] = (double)part;
    __syncthreads();
    double tot = 0;
#pragma unroll
    for (int w = 0; w < NW; ++w) tot += s_wsum[w];
    const float sq = (float)tot, inv = (float)(1.0 / pnorm[ci]);
    for (int pr = tid; pr < NP; pr += T) {
        int ia, jb;
        decode_pair(pr, ia, jb);
        const float f0 = ia != jb ? 1.41421356237309504880f : 2.f;
#pragma unroll
        for (int l = 0; l < L; ++l) {
            const int k = pr * L + l;
            const float g = gs[k];
            gs[k] = (sc.normalise ? (g - qs[k] * sq) * inv : g) * f0 * K[tb.lf + l];
        }
    }
    __syncthreads();
    if (lm >= L2) return;
    const int l = l_of_lm(lm);
    float dreg[NN];
#pragma unroll
    for (int a = 0; a < NN; ++a) dreg[a] = 0.f;
    const float* dp = gs + l;
#pragma unroll
    for (int ia = 0; ia < NN; ++ia)
#pragma unroll
        for (int jb = 0; jb <= ia; ++jb) {
            const float v = dp[(ia * (ia + 1) / 2 + jb) * L];
            dreg[ia] += v * creg[jb];
            if (ia != jb) dreg[jb] += v * creg[ia];
        }
    float* ho = hbuf + (size_t)ci * NS * L2 * NMP;
#pragma unroll
    for (int s = 0; s < NS; ++s) {
        float x[NMP];
#pragma unroll
        for (int a = 0; a < NMP; ++a) {
            const float4* tr = reinterpret_cast<const float4*>(K + tb.Tp + a * NMP);
            float acc = 0.f;
#pragma unroll
            for (int n4 = 0; n4 < NMP / 4; ++n4) {
                const float4 t = tr[n4];
                const float tv[4] = {t.x, t.y, t.z, t.w};
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (4 * n4 + e < NM) acc += tv[e] * dreg[s * NM + 4 * n4 + e];
            }
            x[a] = acc;
        }
        float4* o = reinterpret_cast<float4*>(ho + (size_t)(s * L2 + lm) * NMP);
#pragma unroll
        for (int a4 = 0; a4 < NMP / 4; ++a4) o[a4] = make_float4(x[4 * a4], x[4 * a4 + 1], x[4 * a4 + 2], x[4 * a4 + 3]);
    }
}

template <int L, int NM, int NS>
int launch_bwd_h_lm(gapgpu_context& c, const Coordinate& co, int nc, const SoapConst& sc) {
    constexpr int NN = NS * NM, NPL = NN * (NN + 1) / 2 * L, T = ((L * L + 31) / 32) * 32;
    const size_t sm = sizeof(float) * ((size_t)soap_tab(NM, L).size + 2 * (size_t)((NPL + 3) & ~3));
    GG_CUDA(cudaFuncSetAttribute(k_soap_bwd_h_lm<L, NM, NS>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_soap_bwd_h_lm<L, NM, NS><<<nc, T, sm, c.stream>>>(sc, static_cast<const float*>(co.dtab[1]), nc, c.scratch.as<float>(),
                                                        c.qbuf.as<float>(), c.pnorm.as<double>(), c.Gbuf.as<float>(),
                                                        c.hbuf.as<float>());
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

// a2c[centres[ci]] = ci (the atoms that are no centre keep -1)
__global__ void k_atom_centre(int nc, const int* __restrict__ centres, int* __restrict__ a2c) {
    const int ci = blockIdx.x * blockDim.x + threadIdx.x;
    if (ci < nc) a2c[centres[ci]] = ci;
}

template <int L, int NMP>
__global__ void __launch_bounds__(BP_THREADS, 4) k_soap_bwd_pairs(SoapConst sc, const float* __restrict__ tab, long long npair,
                                                                const int* __restrict__ a2c, const int* __restrict__ ni,
                                                                const int* __restrict__ off, const int* __restrict__ Z,
                                                                const int* __restrict__ nj, const double4* __restrict__ nd,
                                                                const float* __restrict__ hbuf, double* __restrict__ fpair,
                                                                int hsm_floats) {
    constexpr int L2 = L * L, NA2 = NMP / 2;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float* hsm = reinterpret_cast<float*>(smem_raw);
    __shared__ int s_cmin, s_cmax;
    const long long p = blockIdx.x * (long long)BP_THREADS + threadIdx.x;
    const int ai = p < npair ? ni[p] : -1, ci = ai >= 0 ? a2c[ai] : -1;
    // The block's pairs belong to a few consecutive centres, whose h rows are one contiguous
    // range of the buffer: copied into shared memory when it fits, else read through L1.
    const size_t row = (size_t)sc.n_species * L2 * NMP;
    if (threadIdx.x == 0) { s_cmin = INT_MAX; s_cmax = -1; }
    __syncthreads();
    if (ci >= 0) { atomicMin(&s_cmin, ci); atomicMax(&s_cmax, ci); }
    __syncthreads();
    const int cmin = s_cmin, nrow = s_cmax - cmin + 1;
    const bool staged = nrow > 0 && (size_t)nrow * row <= (size_t)hsm_floats;
    if (staged) {
        cp_async_floats(hsm, hbuf + (size_t)cmin * row, (int)(nrow * row));
        cp_async_wait();
    }
    __syncthreads();
    if (ci < 0) return;
    const float* hc = staged ? hsm + (size_t)(ci - cmin) * row : hbuf + (size_t)ci * row;
    if (!staged) {  // the centre's h block into L1, its 128-byte lines shared out over the centre's pairs
        const int p0 = off[ai], cnt = off[ai + 1] - p0, lines = (int)((row * 4 + 127) / 128);
        const char* hb = reinterpret_cast<const char*>(hc);
        for (int k = (int)(p - p0); k < lines; k += cnt) asm volatile("prefetch.L1 [%0];" ::"l"(hb + 128 * (size_t)k));
    }
    const double4 d = nd[p];
    const int s = d.w < sc.rc ? species_channel(sc, Z[nj[p]]) : -1;
    if (s < 0) return;
    const int nm = sc.n_max;
    const SoapTab tb = soap_tab(nm, L);
    const float alpha = (float)sc.alpha;
    const float r = (float)d.w, ir = rinv(r);
    const float ux = (float)d.x * ir, uy = (float)d.y * ir, uz = (float)d.z * ir;
    float f, df;
    cutoff_fn<float>(r, (float)sc.rc, (float)sc.w, f, df);
    const float4* hrow = reinterpret_cast<const float4*>(hc + (size_t)s * L2 * NMP);
    // radial state: rp = rho_{l-1}, rcur = rho_l (pairs of grid points), ix = 1/x, rbv = rb
    float2 rp[NA2], rcur[NA2];
    float ix[NMP], rbv[NMP];
    float e0 = 0.f, h0 = 0.f;  // the rb = 0 grid point, if any (lm = 0 only)
#pragma unroll
    for (int a = 0; a < NMP; ++a) {
        float vm = 0.f, v0 = 0.f, xa = 0.f, rb = 0.f;
        if (a < nm) {
            rb = __ldg(tab + tb.rb + a);
            const float em = rexp(-alpha * (r - rb) * (r - rb));
            if (rb > 0.f) {
                const float ep = rexp(-alpha * (r + rb) * (r + rb));
                xa = rinv(2.f * alpha * r * rb);
                vm = 0.5f * (em + ep) * xa;
                v0 = 0.5f * (em - ep) * xa;
            } else {
                e0 = em;
                h0 = reinterpret_cast<const float*>(hrow)[a];
            }
        }
        ix[a] = xa;
        rbv[a] = rb;
        if (a & 1) { rp[a >> 1].y = vm; rcur[a >> 1].y = v0; }
        else { rp[a >> 1].x = vm; rcur[a >> 1].x = v0; }
    }
    float cm[L], sm[L];
    cm[0] = 1.f;
    sm[0] = 0.f;
#pragma unroll
    for (int m = 1; m < L; ++m) {
        cm[m] = cm[m - 1] * ux - sm[m - 1] * uy;
        sm[m] = sm[m - 1] * ux + cm[m - 1] * uy;
    }
    float q1[L], q2[L], d1[L], d2[L];
#pragma unroll
    for (int m = 0; m < L; ++m) q1[m] = q2[m] = d1[m] = d2[m] = 0.f;
    float Auv = 0.f, Awv = 0.f, Avv = 0.f, Ax = 0.f, Ay = 0.f, Az = 0.f;
    const float t = uz, tar = 2.f * alpha * r;
    // u = sum_a h[lm][a] rho_a, v = sum_a h[lm][a] rb_a rho_{a,l-1}
    auto dots = [&](int lm, const float2* pi, float& u, float& v) {
        float2 uu = make_float2(0.f, 0.f), vv = make_float2(0.f, 0.f);
#pragma unroll
        for (int k = 0; k < NMP / 4; ++k) {
            const float4 h = hrow[lm * (NMP / 4) + k];
            const float2 ha = make_float2(h.x, h.y), hb = make_float2(h.z, h.w);
            uu = __ffma2_rn(ha, rcur[2 * k], uu);
            vv = __ffma2_rn(ha, pi[2 * k], vv);
            uu = __ffma2_rn(hb, rcur[2 * k + 1], uu);
            vv = __ffma2_rn(hb, pi[2 * k + 1], vv);
        }
        u = uu.x + uu.y;
        v = vv.x + vv.y;
    };
#pragma unroll
    for (int l = 0; l < L; ++l) {
        float2 pi[NA2];
#pragma unroll
        for (int k = 0; k < NA2; ++k) pi[k] = make_float2(rbv[2 * k] * rp[k].x, rbv[2 * k + 1] * rp[k].y);
        const int ll = l * l + l;
        float AuvL = 0.f;
#pragma unroll
        for (int m = 0; m <= l; ++m) {
            float q, dq;
            if (m == l) {
                float qmm = 1.f;
#pragma unroll
                for (int k = 1; k <= 2 * m - 1; k += 2) qmm *= (float)k;
                q = qmm;
                dq = 0.f;
            } else if (m == l - 1) {
                q = (float)(2 * m + 1) * t * q1[m];
                dq = (float)(2 * m + 1) * q1[m];
            } else {
                const float ra = c_lra[l * l + m], rbb = c_lrbb[l * l + m];
                q = ra * t * q1[m] - rbb * q2[m];
                dq = ra * (q1[m] + t * d1[m]) - rbb * d2[m];
            }
            q2[m] = q1[m];
            q1[m] = q;
            d2[m] = d1[m];
            d1[m] = dq;
            const float nq = c_lyn[l * l + m] * q, ndq = c_lyn[l * l + m] * dq;
            if (m == 0) {
                float u, v;
                dots(ll, pi, u, v);
                AuvL += nq * u;
                Avv += nq * v;
                Az += ndq * u;
            } else {
                float up, vp, um, vm;
                dots(ll + m, pi, up, vp);
                dots(ll - m, pi, um, vm);
                const float U1 = up * cm[m] + um * sm[m], V1 = vp * cm[m] + vm * sm[m];
                const float Ux = up * cm[m - 1] + um * sm[m - 1], Uy = um * cm[m - 1] - up * sm[m - 1];
                const float am = nq * (float)m;
                AuvL += nq * U1;
                Avv += nq * V1;
                Az += ndq * U1;
                Ax += am * Ux;
                Ay += am * Uy;
            }
        }
        Awv += -(tar + (float)(l + 1) * ir) * AuvL;
        Auv += AuvL;
        // rho_{l+1} = rho_{l-1} - (2l+1) rho_l / x
        const float c2 = (float)(2 * l + 1);
#pragma unroll
        for (int k = 0; k < NA2; ++k) {
            const float2 nx = make_float2(rp[k].x - c2 * ix[2 * k] * rcur[k].x, rp[k].y - c2 * ix[2 * k + 1] * rcur[k].y);
            rp[k] = rcur[k];
            rcur[k] = nx;
        }
    }
    Awv += 2.f * alpha * Avv;
    if (h0 != 0.f) {  // rb = 0: rho_0 = exp(-alpha r^2), d rho_0 / dr = -2 alpha r rho_0, Y_00 constant
        const float y00 = c_lyn[0];
        Auv += h0 * e0 * y00;
        Awv += -tar * h0 * e0 * y00;
    }
    // f = ar u + (I - u u^T) g / r with ar = sum (f w + f' u) Y, g = f sum u dY/du
    const float ar = f * Awv + df * Auv, gx = f * Ax, gy = f * Ay, gz = f * Az;
    const float gu = gx * ux + gy * uy + gz * uz;
    double* fo = fpair + 3 * p;
    fo[0] += (double)(ar * ux + (gx - gu * ux) * ir);
    fo[1] += (double)(ar * uy + (gy - gu * uy) * ir);
    fo[2] += (double)(ar * uz + (gz - gu * uz) * ir);
}

// Forward with the basis sizes fixed at compile time (L = l_max + 1, NMP = n_max padded to
// 4; FP32): the accumulation and the per-centre tail of k_soap_forward, with
//  * the neighbour functions of a chunk computed one thread per staged neighbour with the
//    whole state in registers: warp 0 the radial rows of all grid points (upward Bessel
//    recurrence, l outermost, four grid points per store), warp 1 the Ylm of all (l, m)
//    (the Legendre columns of all m advanced together, constants in constant memory);
//  * one accumulator item per thread: (species, up to three m of one l, four grid points),
//    so each staged radial quadruple feeds up to 12 products;
//  * q, its GEMM-operand copy and c written as vectors.
// Column m of the real spherical harmonics as ylm_column, with m and L fixed at compile
// time: the recurrence constants are constant-memory operands and the loop is unrolled.
__host__ __device__ constexpr float odd_factorial(int m) {
    float q = 1.f;
    for (int k = 1; k <= 2 * m - 1; k += 2) q *= (float)k;
    return q;
}
template <int L, int M>
__device__ __forceinline__ void ylm_col_t(float ux, float uy, float uz, float* Y) {
    float cm = 1.f, sm = 0.f;
#pragma unroll
    for (int k = 0; k < M; ++k) {
        const float c2 = cm * ux - sm * uy;
        sm = sm * ux + cm * uy;
        cm = c2;
    }
    constexpr float qmm = odd_factorial(M);
    float q1 = 0.f, q2 = 0.f;
#pragma unroll
    for (int l = M; l < L; ++l) {
        float q;
        if (l == M) q = qmm;
        else if (l == M + 1) q = (float)(2 * M + 1) * uz * qmm;
        else q = c_lra[l * l + M] * uz * q1 - c_lrbb[l * l + M] * q2;
        q2 = q1;
        q1 = q;
        const float nq = c_lyn[l * l + M] * q;
        if (M == 0) Y[l * l + l] = nq;
        else {
            Y[l * l + l + M] = nq * cm;
            Y[l * l + l - M] = nq * sm;
        }
    }
}
template <int L, int M = 0>
__device__ __forceinline__ void ylm_col_dispatch(int m, float ux, float uy, float uz, float* Y) {
    if constexpr (M < L) {
        if (m == M) ylm_col_t<L, M>(ux, uy, uz, Y);
        else ylm_col_dispatch<L, M + 1>(m, ux, uy, uz, Y);
    }
}

__host__ __device__ constexpr int fwd_triples(int L) {
    int t = 0;
    for (int l = 0; l < L; ++l) t += (2 * l + 1 + 2) / 3;
    return t;
}

template <int L, int NMP>
__global__ void __launch_bounds__(FWD_THREADS, 5) k_soap_fwd_t(SoapConst sc, const float* __restrict__ tab, int nc,
                                                             const int* __restrict__ centres, const int* __restrict__ Z,
                                                             const int* __restrict__ off, const int* __restrict__ nj,
                                                             const double4* __restrict__ nd, float* __restrict__ c_out,
                                                             float* __restrict__ q_out, void* __restrict__ qr_out,
                                                             int qr_half, double* __restrict__ pnorm) {
    constexpr int L2 = L * L, NA4 = NMP / 4, NA2 = NMP / 2, NT = fwd_triples(L);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int ci = blockIdx.x;
    if (ci >= nc) return;
    const int atom = centres[ci];
    const int nm = sc.n_max, NS = sc.n_species;
    const SoapTab tb = soap_tab(nm, L);
    float* K = reinterpret_cast<float*>(smem_raw);
    float* cs = K + tb.size;                          // NS * nm * L2
    float* Ysm = cs + ((NS * nm * L2 + 3) & ~3);      // TC * L2
    float* Ism = Ysm + TC * L2;                       // TC * L * NMP
    float* fcs = Ism + TC * L * NMP;                  // TC
    float* dsm = fcs + TC;                            // TC * DS
    float* ct = Ysm;                                  // NS * L2 * NMP, after the loop
    const int region = fwd_region(sc);
    int* spc = reinterpret_cast<int*>(Ysm + region);  // TC
    int* lst = spc + TC;                              // NS * TC
    int* lcnt = lst + NS * TC;                        // NS
    const int tid = threadIdx.x, bd = blockDim.x;
    copy_to_smem<4>(tab, K, tb.size);
    // this thread's item: species s, lm0 .. lm0 + cnt - 1 (one l), grid points 4 a4 .. 4 a4 + 3
    int own_s = -1, own_l = 0, own_lm0 = 0, own_cnt = 0, own_a4 = 0;
    if (tid < NS * NT * NA4) {
        own_s = tid / (NT * NA4);
        const int rem = tid - own_s * NT * NA4, tr = rem / NA4;
        own_a4 = rem - tr * NA4;
        int k = tr;
        for (int l = 0; l < L; ++l) {
            const int n3 = (2 * l + 1 + 2) / 3;
            if (k < n3) {
                own_l = l;
                own_lm0 = l * l + 3 * k;
                own_cnt = min(3, 2 * l + 1 - 3 * k);
                break;
            }
            k -= n3;
        }
    }
    float acc[3][4];
#pragma unroll
    for (int k = 0; k < 3; ++k) acc[k][0] = acc[k][1] = acc[k][2] = acc[k][3] = 0.f;
    const float alpha = (float)sc.alpha;
    const int p0 = off[atom], p1 = off[atom + 1];
    for (int base = p0; base < p1; base += TC) {
        const int cnt = min(TC, p1 - base);
        __syncthreads();
        {
            ChunkFetch nf;
            nf.load<TC>(base, p1, Z, nj, nd);
            if (tid < 32) build_species_lists<TC>(sc, cnt, nf, spc, lst, lcnt);
            else if (tid - 32 < cnt) {
                const int t = tid - 32;
                stage_neighbour<float>(sc, nf.d, dsm + DS * t, fcs + t, (float*)nullptr);
            }
        }
        __syncthreads();
        {
            // warps 0 .. NA4-1: the radial rows of one quadruple of grid points each; the other
            // warps: Ylm columns m with m mod 2W in {j, 2W-1-j} (W column warps, j = warp - NA4),
            // which gives every column warp the same number of Legendre steps
            const int t = tid & 31, wid = tid >> 5;
            if (t < cnt && spc[t] >= 0) {
                const float* u = dsm + DS * t;
                const float r = u[4], fc = fcs[t];
                if (wid < NA4) {
                    float rp[4], rcur[4], ix[4];
                    bool rb0[4];
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int a = 4 * wid + e;
                        float vm = 0.f, v0 = 0.f, xa = 0.f;
                        rb0[e] = false;
                        if (a < nm) {
                            const float rb = K[tb.rb + a];
                            const float em = rexp(-alpha * (r - rb) * (r - rb));
                            if (rb > 0.f) {
                                const float ep = rexp(-alpha * (r + rb) * (r + rb));
                                xa = rinv(2.f * alpha * r * rb);
                                vm = 0.5f * (em + ep) * xa;
                                v0 = 0.5f * (em - ep) * xa;
                            } else {
                                v0 = em;  // rb = 0: rho_0 = exp(-alpha r^2), rho_l = 0 for l > 0
                                rb0[e] = true;
                            }
                        }
                        rp[e] = vm;
                        rcur[e] = v0;
                        ix[e] = xa;
                    }
                    float4* row = reinterpret_cast<float4*>(Ism + t * L * NMP) + wid;
#pragma unroll
                    for (int l = 0; l < L; ++l) {
                        row[l * NA4] = make_float4(fc * rcur[0], fc * rcur[1], fc * rcur[2], fc * rcur[3]);
                        const float c2 = (float)(2 * l + 1);
#pragma unroll
                        for (int e = 0; e < 4; ++e) {
                            const float nx = rp[e] - c2 * ix[e] * rcur[e];
                            rp[e] = (l == 0 && rb0[e]) ? 0.f : rcur[e];
                            rcur[e] = nx;
                        }
                    }
                } else {
                    const int j = wid - NA4, W2 = 2 * (FWD_THREADS / 32 - NA4);
                    for (int m = 0; m < L; ++m) {
                        const int mm = m % W2;
                        if (mm == j || mm == W2 - 1 - j) ylm_col_dispatch<L>(m, u[0], u[1], u[2], Ysm + t * L2);
                    }
                }
            }
        }
        __syncthreads();
        if (own_s >= 0) {
            const int nt = lcnt[own_s];
            const int* ls = lst + own_s * TC;
            for (int qq = 0; qq < nt; ++qq) {
                const int t = ls[qq];
                const float4 rho = *reinterpret_cast<const float4*>(Ism + (t * L + own_l) * NMP + 4 * own_a4);
                const float* yv = Ysm + t * L2 + own_lm0;
#pragma unroll
                for (int k = 0; k < 3; ++k)
                    if (k < own_cnt) {
                        const float y = yv[k];
                        acc[k][0] += y * rho.x;
                        acc[k][1] += y * rho.y;
                        acc[k][2] += y * rho.z;
                        acc[k][3] += y * rho.w;
                    }
            }
        }
    }
    __syncthreads();  // the staging area becomes ct
    if (own_s >= 0) {
#pragma unroll
        for (int k = 0; k < 3; ++k)
            if (k < own_cnt)
                *reinterpret_cast<float4*>(ct + (own_s * L2 + own_lm0 + k) * NMP + 4 * own_a4) =
                    make_float4(acc[k][0], acc[k][1], acc[k][2], acc[k][3]);
    }
    __syncthreads();
    // c[s][n][lm] = sum_a T_an ct[s][lm][a]  (+ central atom at l = 0): one thread per (s, lm)
    const int zc = Z[atom];
    for (int k = tid; k < NS * L2; k += bd) {
        const int s = k / L2, lm = k - s * L2;
        const float4* v4 = reinterpret_cast<const float4*>(ct + (s * L2 + lm) * NMP);
        float va[NMP];
#pragma unroll
        for (int a4 = 0; a4 < NA4; ++a4) {
            const float4 w = v4[a4];
            va[4 * a4] = w.x; va[4 * a4 + 1] = w.y; va[4 * a4 + 2] = w.z; va[4 * a4 + 3] = w.w;
        }
        const bool centre = lm == 0 && (sc.centre_all || sc.species_Z[s] == zc || sc.species_Z[s] == 0);
        for (int n = 0; n < nm; ++n) {
            const float4* tr = reinterpret_cast<const float4*>(K + tb.Tt + n * NMP);
            float x = 0.f;
#pragma unroll
            for (int a4 = 0; a4 < NA4; ++a4) {
                const float4 w = tr[a4];
                x += w.x * va[4 * a4] + w.y * va[4 * a4 + 1] + w.z * va[4 * a4 + 2] + w.w * va[4 * a4 + 3];
            }
            if (centre) x += K[tb.cr + n];
            cs[(s * nm + n) * L2 + lm] = x;
        }
    }
    __syncthreads();
    {
        float* cg = c_out + (size_t)ci * sc.ncomp;
        if ((sc.ncomp & 3) == 0) {
            for (int k = tid; k < sc.ncomp / 4; k += bd)
                reinterpret_cast<float4*>(cg)[k] = reinterpret_cast<const float4*>(cs)[k];
        } else {
            for (int k = tid; k < sc.ncomp; k += bd) cg[k] = cs[k];
        }
    }
    // power spectrum: one item per (l, 2x2 block of channel rows (ia, jb), ia >= jb)
    float* ps = Ysm;
    float ssr = 0.f;
    {
        const int NR = NS * nm, NB = (NR + 1) / 2, nblk = NB * (NB + 1) / 2;
        if (tid < nblk * L) {
            Walk2 w(tid, bd, nblk);
            for (; w.i < L; w.next()) {
                const int l = w.i;
                int bi = (int)((sqrtf((float)(8 * w.j + 1)) - 1.0f) * 0.5f);
                while ((bi + 1) * (bi + 2) / 2 <= w.j) ++bi;
                while (bi * (bi + 1) / 2 > w.j) --bi;
                const int bj = w.j - bi * (bi + 1) / 2;
                const int i0 = 2 * bi, j0 = 2 * bj;
                const bool i1ok = i0 + 1 < NR, j1ok = j0 + 1 < NR;
                const float* a0 = cs + i0 * L2 + l * l;
                const float* a1 = cs + (i1ok ? i0 + 1 : i0) * L2 + l * l;
                const float* b0 = cs + j0 * L2 + l * l;
                const float* b1 = cs + (j1ok ? j0 + 1 : j0) * L2 + l * l;
                float v00 = 0.f, v01 = 0.f, v10 = 0.f, v11 = 0.f;
                for (int m = 0; m < 2 * l + 1; ++m) {
                    const float x0 = a0[m], x1 = a1[m], y0 = b0[m], y1 = b1[m];
                    v00 += x0 * y0;
                    v01 += x0 * y1;
                    v10 += x1 * y0;
                    v11 += x1 * y1;
                }
                const float lf = K[tb.lf + l], r2 = 1.41421356237309504880f;
                auto put = [&](int ia, int jb, float v) {
                    v *= (ia != jb ? r2 : 1.f) * lf;
                    ps[(ia * (ia + 1) / 2 + jb) * L + l] = v;
                    ssr += v * v;
                };
                put(i0, j0, v00);
                if (j1ok && bi != bj) put(i0, j0 + 1, v01);
                if (i1ok) put(i0 + 1, j0, v10);
                if (i1ok && j1ok) put(i0 + 1, j0 + 1, v11);
            }
        }
    }
    __shared__ double s_wsum[FWD_THREADS / 32];
    __shared__ float s_inv;
    ssr = warp_sum(ssr);
    if ((tid & 31) == 0) s_wsum[tid >> 5] = (double)ssr;
    __syncthreads();
    if (tid == 0) {
        double tot = 0;
        for (int w = 0; w < FWD_THREADS / 32; ++w) tot += s_wsum[w];
        const double nrm = sqrt(tot);
        pnorm[ci] = nrm;
        s_inv = sc.normalise ? (float)(1.0 / nrm) : 1.f;
    }
    __syncthreads();
    const float inv = s_inv, sig = (float)sc.sigma0;
    const int np = sc.n_pairs * L;
    float* qg = q_out + (size_t)ci * sc.dpad;
    float* qrg = qr_out && !qr_half ? static_cast<float*>(qr_out) + (size_t)ci * sc.dpad : nullptr;
    __half* qhg = qr_out && qr_half ? static_cast<__half*>(qr_out) + (size_t)ci * sc.dpad : nullptr;
    for (int k4 = tid; k4 < sc.dpad / 4; k4 += bd) {  // dpad is a multiple of 4
        float v[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int k = 4 * k4 + e;
            v[e] = k < np ? ps[k] * inv : (k == np ? sig : 0.f);
        }
        reinterpret_cast<float4*>(qg)[k4] = make_float4(v[0], v[1], v[2], v[3]);
        if (qrg)
            __stcs(reinterpret_cast<float4*>(qrg) + k4,
                   make_float4(round_tf32(v[0]), round_tf32(v[1]), round_tf32(v[2]), round_tf32(v[3])));
        if (qhg) {
            const __half2 h0 = __floats2half2_rn(v[0], v[1]), h1 = __floats2half2_rn(v[2], v[3]);
            uint2 pk;
            pk.x = *reinterpret_cast<const unsigned*>(&h0);
            pk.y = *reinterpret_cast<const unsigned*>(&h1);
            reinterpret_cast<uint2*>(qhg)[k4] = pk;
        }
    }
}

template <int L, int NMP>
int launch_fwd_t(gapgpu_context& c, const Coordinate& co, int nc, const SoapConst& sc, size_t sm) {
    GG_CUDA(cudaFuncSetAttribute(k_soap_fwd_t<L, NMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_soap_fwd_t<L, NMP><<<nc, FWD_THREADS, sm, c.stream>>>(
        sc, static_cast<const float*>(co.dtab[1]), nc, c.cur_centres, c.Z.as<int>(), c.nbr_off.as<int>(), c.nbr_j.as<int>(),
        c.nbr_d.as<double4>(), c.scratch.as<float>(), c.qbuf.as<float>(),
        c.precision == GAPGPU_MIXED_TF32 ? c.qlo.p : nullptr, gemm1_f16_active(c, co) ? 1 : 0, c.pnorm.as<double>());
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

// The fixed-size FP32 forward where it has an instance (-1 otherwise).
int forward_fixed(gapgpu_context& c, const Coordinate& co, int nc, const SoapConst& sc, size_t sm) {
    const int L = sc.l_max + 1, NMP = nmp_of(sc.n_max);
    if ((sc.dpad & 3) != 0) return -1;
    auto fits = [&](int T, int na4) { return sc.n_species * T * na4 <= FWD_THREADS; };
    if (L == 9 && NMP == 12 && fits(fwd_triples(9), 3)) return launch_fwd_t<9, 12>(c, co, nc, sc, sm);
    if (L == 7 && NMP == 8 && fits(fwd_triples(7), 2)) return launch_fwd_t<7, 8>(c, co, nc, sc, sm);
    if (L == 5 && NMP == 8 && fits(fwd_triples(5), 2)) return launch_fwd_t<5, 8>(c, co, nc, sc, sm);
    if (L == 5 && NMP == 4 && fits(fwd_triples(5), 1)) return launch_fwd_t<5, 4>(c, co, nc, sc, sm);
    return -1;
}

__global__ void k_centre_flags(int n, const int* __restrict__ Z, const int* __restrict__ mask, SoapConst sc, int nZ,
                               const int* __restrict__ zlist, int* __restrict__ flags) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    int ok = 0;
    for (int k = 0; k < nZ; ++k) if (zlist[k] == Z[a] || zlist[k] == 0) ok = 1;
    if (mask && !mask[a]) ok = 0;
    flags[a] = ok;
}

__global__ void k_iota(int n, int* out) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) out[a] = a;
}

template <class R>
size_t fwd_smem(const SoapConst& sc) {
    const int L = sc.l_max + 1, L2 = L * L, NS = sc.n_species;
    return sizeof(R) * ((size_t)soap_tab(sc.n_max, L).size + (size_t)((NS * sc.n_max * L2 + 3) & ~3) + fwd_region(sc)) +
           sizeof(int) * (TC + NS * TC + NS) + (size_t)L2 + 2 + 2 * (size_t)sc.n_pairs + 64;
}
template <class R>
size_t bwd_smem(const SoapConst& sc) {
    const int L = sc.l_max + 1;
    return sizeof(R) * (size_t)bwd_plan(sc).ints_at + sizeof(int) * (TCB + sc.n_species * TCB + sc.n_species) +
           (size_t)((L * L + 1) & ~1) + 2 * (size_t)sc.n_pairs + 64;
}

template <class R, int FQ>
int launch_forward_fq(gapgpu_context& c, const Coordinate& co, int nc, const SoapConst& sc, size_t sm) {
    GG_CUDA(cudaFuncSetAttribute(k_soap_forward<R, FQ>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const R* tab = static_cast<const R*>(co.dtab[sizeof(R) == 4 ? 1 : 0]);
    k_soap_forward<R, FQ><<<nc, FWD_THREADS, sm, c.stream>>>(sc, tab, nc, c.cur_centres, c.Z.as<int>(), c.nbr_off.as<int>(),
                                                             c.nbr_j.as<int>(), c.nbr_d.as<double4>(), c.scratch.as<R>(),
                                                             c.qbuf.as<R>(),
                                                             c.precision == GAPGPU_MIXED_TF32 ? c.qlo.p : nullptr,
                                                             gemm1_f16_active(c, co) ? 1 : 0,
                                                             c.pnorm.as<double>());
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

template <class R>
int launch_forward(gapgpu_context& c, const Coordinate& co, int nc) {
    SoapConst sc = soap_const(co);
    size_t sm = fwd_smem<R>(sc);
    if (sm > 200 * 1024) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "SOAP basis too large for the shared-memory forward kernel");
    if (sizeof(R) == 4 && c.soap_fwd_fixed) {
        const int rc = forward_fixed(c, co, nc, sc, sm);
        if (rc >= 0) return rc;
    }
    const int items = sc.n_species * (sc.l_max + 1) * (sc.l_max + 1) * (nmp_of(sc.n_max) / 4);
    if (items <= FQ_SMALL * FWD_THREADS) return launch_forward_fq<R, FQ_SMALL>(c, co, nc, sc, sm);
    if (items <= FQ_LARGE * FWD_THREADS) return launch_forward_fq<R, FQ_LARGE>(c, co, nc, sc, sm);
    GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "SOAP basis too large for the forward kernel's register accumulators");
}

template <int L, int NMP>
int launch_bwd_pairs(gapgpu_context& c, const Coordinate& co, const SoapConst& sc) {
    const long long P = c.n_pairs;
    if (P == 0) return GAPGPU_OK;
    const unsigned nb = (unsigned)((P + BP_THREADS - 1) / BP_THREADS);
    const int hsm_floats = BP_SMEM_BYTES / (int)sizeof(float);
    GG_CUDA(cudaFuncSetAttribute(k_soap_bwd_pairs<L, NMP>, cudaFuncAttributeMaxDynamicSharedMemorySize, BP_SMEM_BYTES));
    k_soap_bwd_pairs<L, NMP><<<nb, BP_THREADS, BP_SMEM_BYTES, c.stream>>>(sc, static_cast<const float*>(co.dtab[1]), P, c.a2c.as<int>(),
                                                              c.nbr_i.as<int>(), c.nbr_off.as<int>(), c.Z.as<int>(),
                                                              c.nbr_j.as<int>(),
                                                              c.nbr_d.as<double4>(), c.hbuf.as<float>(),
                                                              c.fpair.as<double>(), hsm_floats);
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

// The two-kernel FP32 backward for the basis sizes the pair kernel is compiled for; -1
// where it has no instance (the block kernel runs instead).
int backward_split(gapgpu_context& c, const Coordinate& co, int n, int nc) {
    const SoapConst sc = soap_const(co);
    const int NN = sc.n_species * sc.n_max, L = sc.l_max + 1, NMP = nmp_of(sc.n_max);
    if (NN > BH_MAXNN || sc.n_pairs != NN * (NN + 1) / 2) return -1;
    int (*pairs)(gapgpu_context&, const Coordinate&, const SoapConst&) = nullptr;
    if (L == 9 && NMP == 12) pairs = launch_bwd_pairs<9, 12>;
    else if (L == 7 && NMP == 8) pairs = launch_bwd_pairs<7, 8>;
    else if (L == 5 && NMP == 8) pairs = launch_bwd_pairs<5, 8>;
    else if (L == 5 && NMP == 4) pairs = launch_bwd_pairs<5, 4>;
    if (!pairs) return -1;
    const size_t sm = sizeof(float) * bh_floats(sc);
    if (sm > 200 * 1024) return -1;
    int rc;
    if ((rc = c.hbuf.ensure(sizeof(float) * (size_t)nc * sc.n_species * L * L * NMP)) ||
        (rc = c.a2c.ensure(sizeof(int) * (size_t)n)))
        return rc;
    const int nm = sc.n_max, ns = sc.n_species;
    if (L == 9 && nm == 10 && ns == 2) rc = launch_bwd_h_lm<9, 10, 2>(c, co, nc, sc);
    else if (L == 7 && nm == 8 && ns == 1) rc = launch_bwd_h_lm<7, 8, 1>(c, co, nc, sc);
    else if (L == 5 && nm == 4 && ns == 2) rc = launch_bwd_h_lm<5, 4, 2>(c, co, nc, sc);
    else {
        GG_CUDA(cudaFuncSetAttribute(k_soap_bwd_h, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
        k_soap_bwd_h<<<nc, BH_THREADS, sm, c.stream>>>(sc, static_cast<const float*>(co.dtab[1]), nc, c.scratch.as<float>(),
                                                       c.qbuf.as<float>(), c.pnorm.as<double>(), c.Gbuf.as<float>(),
                                                       c.hbuf.as<float>());
        c.launches++;
    }
    if (rc) return rc;
    GG_CUDA(cudaMemsetAsync(c.a2c.p, 0xff, sizeof(int) * (size_t)n, c.stream));
    k_atom_centre<<<(nc + 255) / 256, 256, 0, c.stream>>>(nc, c.cur_centres, c.a2c.as<int>());
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return pairs(c, co, sc);
}

template <class R>
int launch_backward(gapgpu_context& c, const Coordinate& co, int n, int nc) {
    if (sizeof(R) == 4 && c.soap_bwd_nb) {
        const int rc = backward_split(c, co, n, nc);
        if (rc >= 0) return rc;
    }
    SoapConst sc = soap_const(co);
    size_t sm = bwd_smem<R>(sc);
    if (sm > 200 * 1024) GG_FAIL(GAPGPU_ERR_UNSUPPORTED, "SOAP basis too large for the shared-memory backward kernel");
    GG_CUDA(cudaFuncSetAttribute(k_soap_backward<R>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    const R* tab = static_cast<const R*>(co.dtab[sizeof(R) == 4 ? 1 : 0]);
    k_soap_backward<R><<<nc, BWD_THREADS, sm, c.stream>>>(sc, tab, nc, c.cur_centres, c.Z.as<int>(),
                                                          c.nbr_off.as<int>(), c.nbr_j.as<int>(), c.nbr_d.as<double4>(),
                                                          c.scratch.as<R>(), c.qbuf.as<R>(), c.pnorm.as<double>(),
                                                          c.Gbuf.as<R>(), c.fpair.as<double>());
    c.launches++;
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

}  // namespace

int upload_soap_tables(Coordinate& co) {
    const SoapParams& sp = co.soap;
    const int nm = sp.n_max, L = sp.l_max + 1;
    const SoapTab tb = soap_tab(nm, L);
    std::vector<double> h(tb.size, 0.0);
    const int NMP = nmp_of(nm);
    for (int k = 0; k < nm * nm; ++k) h[tb.T + k] = sp.T[k];
    for (int a = 0; a < nm; ++a)
        for (int n = 0; n < nm; ++n) {
            h[tb.Tt + n * NMP + a] = sp.T[a * nm + n];
            h[tb.Tp + a * NMP + n] = sp.T[a * nm + n];
        }
    for (int a = 0; a < nm; ++a) { h[tb.rb + a] = sp.rb[a]; h[tb.cr + a] = sp.centre_R[a]; }
    for (int l = 0; l < L; ++l) {
        h[tb.lf + l] = 1.0 / std::sqrt((double)(2 * l + 1));
        for (int m = 0; m <= l; ++m) {
            double lf = 1.0;
            for (int k = l - m + 1; k <= l + m; ++k) lf /= k;
            const double N = std::sqrt((2 * l + 1) / (4.0 * M_PI) * lf);
            h[tb.yn + l * l + m] = m == 0 ? N : std::sqrt(2.0) * N;
            if (l >= m + 2) {
                h[tb.ra + l * l + m] = (double)(2 * l - 1) / (double)(l - m);
                h[tb.rbb + l * l + m] = (double)(l + m - 1) / (double)(l - m);
            }
        }
    }
    std::vector<float> f(h.begin(), h.end());
    {  // the Legendre constants of the pair kernel for every l <= MAX_LMAX (model independent)
        static std::once_flag once;
        static int once_rc = GAPGPU_OK;
        std::call_once(once, [] {
            float ra[MAX_L2] = {}, rbb[MAX_L2] = {}, yn[MAX_L2] = {};
            for (int l = 0; l <= MAX_LMAX; ++l)
                for (int m = 0; m <= l; ++m) {
                    double lf = 1.0;
                    for (int k = l - m + 1; k <= l + m; ++k) lf /= k;
                    const double N = std::sqrt((2 * l + 1) / (4.0 * M_PI) * lf);
                    yn[l * l + m] = (float)(m == 0 ? N : std::sqrt(2.0) * N);
                    if (l >= m + 2) {
                        ra[l * l + m] = (float)((double)(2 * l - 1) / (double)(l - m));
                        rbb[l * l + m] = (float)((double)(l + m - 1) / (double)(l - m));
                    }
                }
            if (cudaMemcpyToSymbol(c_lra, ra, sizeof(ra)) != cudaSuccess || cudaMemcpyToSymbol(c_lrbb, rbb, sizeof(rbb)) != cudaSuccess ||
                cudaMemcpyToSymbol(c_lyn, yn, sizeof(yn)) != cudaSuccess)
                once_rc = GAPGPU_ERR_CUDA;
        });
        if (once_rc != GAPGPU_OK) GG_FAIL(GAPGPU_ERR_CUDA, "uploading the Legendre constants failed");
    }
    GG_CUDA(cudaMalloc(&co.dtab[0], sizeof(double) * h.size()));
    GG_CUDA(cudaMalloc(&co.dtab[1], sizeof(float) * f.size()));
    GG_CUDA(cudaMemcpy(co.dtab[0], h.data(), sizeof(double) * h.size(), cudaMemcpyHostToDevice));
    GG_CUDA(cudaMemcpy(co.dtab[1], f.data(), sizeof(float) * f.size(), cudaMemcpyHostToDevice));
    return GAPGPU_OK;
}

int select_centres(gapgpu_context& c, const Coordinate& co, int n, const int* d_mask, int* nc_out) {
    int rc;
    if ((rc = c.flags.ensure(sizeof(int) * n)) || (rc = c.ncent.ensure(sizeof(int) * 2)) ||
        (rc = c.eatom.ensure(sizeof(double) * n)))
        return rc;
    SoapConst sc = soap_const(co);
    int zl[MAX_CENTRE_Z];
    for (int k = 0; k < co.soap.n_Z; ++k) zl[k] = co.soap.Z[k];
    int* dz = c.ncent.as<int>();
    (void)dz;
    // small Z list through a kernel argument copy
    if ((rc = c.minmax.ensure(sizeof(int) * MAX_CENTRE_Z + 64))) return rc;
    GG_CUDA(cudaMemcpyAsync(c.minmax.p, zl, sizeof(int) * co.soap.n_Z, cudaMemcpyHostToDevice, c.stream));
    const int TB = 256, nb = (n + TB - 1) / TB;
    k_centre_flags<<<nb, TB, 0, c.stream>>>(n, c.Z.as<int>(), d_mask, sc, co.soap.n_Z, c.minmax.as<int>(), c.flags.as<int>());
    k_iota<<<nb, TB, 0, c.stream>>>(n, c.atom_idx.as<int>());
    c.launches += 2;
    size_t tmp = 0;
    cub::DeviceSelect::Flagged(nullptr, tmp, c.atom_idx.as<int>(), c.flags.as<int>(), c.cur_centres, c.ncent.as<int>(),
                               n, c.stream);
    if ((rc = c.cub_tmp.ensure(tmp))) return rc;
    GG_CUDA(cub::DeviceSelect::Flagged(c.cub_tmp.p, tmp, c.atom_idx.as<int>(), c.flags.as<int>(), c.cur_centres,
                                       c.ncent.as<int>(), n, c.stream));
    int nc = 0;
    GG_CUDA(cudaMemcpyAsync(&nc, c.ncent.p, sizeof(int), cudaMemcpyDeviceToHost, c.stream));
    GG_CUDA(cudaStreamSynchronize(c.stream));
    *nc_out = nc;
    return GAPGPU_OK;
}

int soap_forward(gapgpu_context& c, const Coordinate& co, int n, int nc) {
    (void)n;
    SoapConst sc = soap_const(co);
    const bool mixed = c.precision != GAPGPU_FP64;
    const size_t rs = mixed ? sizeof(float) : sizeof(double);
    int rc;
    if ((rc = c.scratch.ensure(rs * (size_t)nc * sc.ncomp)) || (rc = c.qbuf.ensure(rs * (size_t)nc * sc.dpad)) ||
        (rc = c.pnorm.ensure(sizeof(double) * nc)))
        return rc;
    if (c.precision == GAPGPU_MIXED_TF32 && (rc = c.qlo.ensure(sizeof(float) * (size_t)nc * sc.dpad))) return rc;
    if (nc == 0) return GAPGPU_OK;
    return mixed ? launch_forward<float>(c, co, nc) : launch_forward<double>(c, co, nc);
}

int soap_backward(gapgpu_context& c, const Coordinate& co, int n, int nc) {
    (void)n;
    if (nc == 0) return GAPGPU_OK;
    return c.precision != GAPGPU_FP64 ? launch_backward<float>(c, co, n, nc) : launch_backward<double>(c, co, n, nc);
}

}  // namespace gapgpu
