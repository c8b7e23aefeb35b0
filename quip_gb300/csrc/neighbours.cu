// neighbours.cu -- K1: cell-list neighbour build with QUIP's semantics.
//
// Restates connection_calc_connect (src/libAtoms/Connection.f95:1035-1310) for the GPU:
//   * atoms are wrapped into the (effective) cell by map_shift = -floor(s + 0.5)
//     (partition_atoms :1519-1587) and binned with cell_of_pos (:1589-1621);
//   * cells per axis from divide_cell (:1674-1691), image range per axis from
//     fit_box_in_cell (:2204-2237) reduced to max(1, (N+1)/2) (:1145-1151), clipped
//     for non-periodic axes as get_min_max_images (:1448-1513);
//   * a pair (i, j, shift) is kept when |r_j + L shift - r_i| < cutoff (strict,
//     test_form_bond :517); there is NO minimum-image convention, every periodic image
//     inside the cutoff is its own entry, and only the exact self at zero shift in the
//     same cell is skipped (:1265-1270);
//   * pair shift = cell-image shift - map_shift_i + map_shift_j (:1273-1276).
// The reference builds a half list (atom1 <= atom2) and exposes both directions
// through neighbour1/neighbour2.  The image ranges are symmetric, so every atom's
// full list is exactly the set the reference iterates; here each atom scans its own
// image cells and emits its full list directly (no atomics: count, scan, fill).
// Atoms are sorted by cell with a stable radix sort so that each list has a fixed,
// reproducible order (cell-image loop order, then atom index).
//
// Batches: many independent structures are built in one pass.  Each structure has its
// own geometry record (lattice, cell grid, image ranges) and a block of global cell
// indices, so atoms of different structures never share a cell and one sort and one
// pair pass serve the whole batch.  A single structure is a batch of one.
//
// Skin reuse (Connection.f95:1086-1125, :1321-1445): a list built at cutoff + skin is
// kept while every atom has moved less than skin/2 since the build; only the pair
// displacements are recomputed (k_distances, the same formula as the fill pass).
#include <cub/cub.cuh>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <mutex>

#include "context.h"

namespace gapgpu {

namespace {

__device__ __forceinline__ int pack_shift(int a, int b, int c) {
    return ((a + 512) & 1023) | (((b + 512) & 1023) << 10) | (((c + 512) & 1023) << 20);
}

__device__ __forceinline__ int sid_of(const int* __restrict__ sid, int a) { return sid ? sid[a] : 0; }

// pair displacement d = pos_b - pos_a + L shift, FP64 without fused multiply-add
// (the order of test_form_bond), and r = |d|.
__device__ __forceinline__ void pair_vector(const double* __restrict__ pos, const double* lat, int a, int b, int s0, int s1,
                                            int s2, double& d0, double& d1, double& d2, double& r) {
    d0 = __dsub_rn(pos[3 * b], pos[3 * a]); d1 = __dsub_rn(pos[3 * b + 1], pos[3 * a + 1]);
    d2 = __dsub_rn(pos[3 * b + 2], pos[3 * a + 2]);
    d0 = __dadd_rn(d0, __dmul_rn(lat[0], (double)s0)); d1 = __dadd_rn(d1, __dmul_rn(lat[1], (double)s0));
    d2 = __dadd_rn(d2, __dmul_rn(lat[2], (double)s0));
    d0 = __dadd_rn(d0, __dmul_rn(lat[3], (double)s1)); d1 = __dadd_rn(d1, __dmul_rn(lat[4], (double)s1));
    d2 = __dadd_rn(d2, __dmul_rn(lat[5], (double)s1));
    d0 = __dadd_rn(d0, __dmul_rn(lat[6], (double)s2)); d1 = __dadd_rn(d1, __dmul_rn(lat[7], (double)s2));
    d2 = __dadd_rn(d2, __dmul_rn(lat[8], (double)s2));
    r = sqrt(__dadd_rn(__dadd_rn(__dmul_rn(d0, d0), __dmul_rn(d1, d1)), __dmul_rn(d2, d2)));
}

// Error-free transformations (Knuth's TwoSum; TwoProd with a fused multiply-add),
// written with round-to-nearest intrinsics so that the compiler neither fuses nor
// reorders them.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// One component of d = pos_b - pos_a + L s in FP32, each position and lattice entry
// carried as hi + lo floats: the large terms are summed exactly (TwoSum/TwoProd) and
// the small ones added to the error, so d is accurate to about one FP32 ulp of |d|
// even when the positions are far from the origin.
__device__ __forceinline__ float eft_component(float bh, float bl, float ah, float al, const float* Lh, const float* Ll,
                                               float s0, float s1, float s2) {
    float hi, e, err;
    two_sum(bh, -ah, hi, err);
    const float sk[3] = {s0, s1, s2};
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float p = __fmul_rn(Lh[3 * k], sk[k]);
        const float ep = __fmaf_rn(Lh[3 * k], sk[k], -p);
        two_sum(hi, p, hi, e);
        err += e + ep + Ll[3 * k] * sk[k];
    }
    return hi + (err + (bl - al));
}

__device__ __forceinline__ void pair_vector_mixed(const float4* __restrict__ phi, const float4* __restrict__ plo,
                                                  const GeomDev& g, int a, int b, int s0, int s1, int s2, double& d0,
                                                  double& d1, double& d2, double& r) {
    const float4 ah = phi[a], al = plo[a], bh = phi[b], bl = plo[b];
    const float f0 = (float)s0, f1 = (float)s1, f2 = (float)s2;
    const float x = eft_component(bh.x, bl.x, ah.x, al.x, g.lat32, g.lat_lo, f0, f1, f2);
    const float y = eft_component(bh.y, bl.y, ah.y, al.y, g.lat32 + 1, g.lat_lo + 1, f0, f1, f2);
    const float z = eft_component(bh.z, bl.z, ah.z, al.z, g.lat32 + 2, g.lat_lo + 2, f0, f1, f2);
    d0 = x;
    d1 = y;
    d2 = z;
    r = sqrtf(x * x + y * y + z * z);
}

// Positions as hi + lo floats for the mixed path's displacements.
__global__ void k_split_pos(int n, const double* __restrict__ pos, float4* __restrict__ phi, float4* __restrict__ plo) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const double x = pos[3 * a], y = pos[3 * a + 1], z = pos[3 * a + 2];
    const float hx = (float)x, hy = (float)y, hz = (float)z;
    phi[a] = make_float4(hx, hy, hz, 0.f);
    plo[a] = make_float4((float)(x - hx), (float)(y - hy), (float)(z - hz), 0.f);
}

__global__ void k_assign(int n, const double* __restrict__ pos, const GeomDev* __restrict__ geoms,
                         const int* __restrict__ sid, int* __restrict__ key, int* __restrict__ idx, int* __restrict__ ms,
                         int* __restrict__ bad) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    const GeomDev& g = geoms[sid_of(sid, a)];
    double p[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
    if (!(isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]))) atomicOr(bad, 1);
    int c3[3];
    for (int d = 0; d < 3; ++d) {
        double lp = g.lat_eff_inv[d] * p[0] + g.lat_eff_inv[3 + d] * p[1] + g.lat_eff_inv[6 + d] * p[2] - g.lat_off[d];
        int m = g.pbc[d] ? -(int)floor(lp + 0.5) : 0;
        ms[3 * a + d] = m;
        double t = lp + m;
        int ci = (int)floor((double)g.cellsN[d] * (t + 0.5)) + 1;
        ci = ci < 1 ? 1 : (ci > g.cellsN[d] ? g.cellsN[d] : ci);
        c3[d] = ci - 1;
    }
    key[a] = g.cell_base + c3[0] + g.cellsN[0] * (c3[1] + g.cellsN[1] * c3[2]);
    idx[a] = a;
}

// Wrapped positions (pos + L map_shift - origin) in FP32, in cell-sorted order, for the
// pre-filter: magnitudes stay within the cell, so FP32 rounding is ~1e-7 of the cell size.
__global__ void k_wrapped(int n, const double* __restrict__ pos, const GeomDev* __restrict__ geoms,
                          const int* __restrict__ sid, const int* __restrict__ sorted, const int* __restrict__ ms,
                          float4* __restrict__ wpos) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int a = sorted[k];
    const GeomDev& g = geoms[sid_of(sid, a)];
    double p[3];
    for (int d = 0; d < 3; ++d)
        p[d] = pos[3 * a + d] + g.lat[d] * ms[3 * a] + g.lat[3 + d] * ms[3 * a + 1] + g.lat[6 + d] * ms[3 * a + 2] - g.origin[d];
    wpos[k] = make_float4((float)p[0], (float)p[1], (float)p[2], 0.f);
}

__global__ void k_cell_ranges(int n, const int* __restrict__ key, int* __restrict__ start, int* __restrict__ end) {
    int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    int c = key[k];
    if (k == 0 || key[k - 1] != c) start[c] = k;
    if (k == n - 1 || key[k + 1] != c) end[c] = k + 1;
}

// One warp per atom (atoms taken in cell order for locality).  The warp walks the
// atom's image cells in the reference's loop order; lanes take the candidates of a
// cell 32 at a time, so the emitted order (cell-image order, then position in the
// sorted cell) is fixed.  A candidate is first measured in FP32 on wrapped coordinates,
// whose error is far below the margin: beyond cutoff + margin it is out, inside
// cutoff - margin it is in.  Only the thin band between is decided by the exact FP64
// test of test_form_bond (dd = pos_b - pos_a + L shift accumulated without fused
// multiply-add, kept when sqrt(dd.dd) < cutoff).  Count and fill take the same
// decisions; the fill pass computes the FP64 displacement of every kept pair.
// CALLER_LAYOUT (fill only): write just j and the unpacked shift (3 ints per entry)
// into caller-owned arrays, the layout of gapgpu_neighbours; nd/ni are not written.
// MIXED (fill only): kept pairs outside the band take their displacement from the FP32
// error-free arithmetic of pair_vector_mixed instead of FP64.
template <bool FILL, bool CALLER_LAYOUT = false, bool MIXED = false>
__global__ void __launch_bounds__(128) k_pairs(int n, const double* __restrict__ pos, const float4* __restrict__ wpos,
                                               const float4* __restrict__ phi, const float4* __restrict__ plo,
                                               const GeomDev* __restrict__ geoms, const int* __restrict__ sid,
                                               const int* __restrict__ key_of_atom, const int* __restrict__ ms,
                                               const int* __restrict__ sorted, const int* __restrict__ cstart,
                                               const int* __restrict__ cend, int* __restrict__ cnt,
                                               const int* __restrict__ off, int* __restrict__ nj, double4* __restrict__ nd,
                                               int* __restrict__ ns, int* __restrict__ ni, int* __restrict__ bad) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= n) return;
    const int a = sorted[warp];
    const GeomDev& g = geoms[sid_of(sid, a)];
    const float4 pa32 = wpos[warp];
    const int lin = key_of_atom[a] - g.cell_base;
    int cc[3] = {lin % g.cellsN[0], (lin / g.cellsN[0]) % g.cellsN[1], lin / (g.cellsN[0] * g.cellsN[1])};
    int mn[3], mx[3];
    for (int d = 0; d < 3; ++d) {
        int c1 = cc[d] + 1;  // 1-based as in the reference
        if (g.pbc[d]) { mn[d] = -g.img[d]; mx[d] = g.img[d]; }
        else {
            mn[d] = (g.img[d] < c1) ? -g.img[d] : -c1 + 1;
            mx[d] = (g.img[d] < g.cellsN[d] - c1) ? g.img[d] : g.cellsN[d] - c1;
        }
    }
    const int msa0 = ms[3 * a], msa1 = ms[3 * a + 1], msa2 = ms[3 * a + 2];
    const float lim2 = g.lim2, sure2 = g.sure2;
    const double cutoff = g.cutoff;
    int count = 0;
    const int base = FILL ? off[a] : 0;
    const unsigned lt = (1u << lane) - 1u, full = 0xffffffffu;
    // The image cells in (k, j, i) order, i fastest, 32 at a time: lane c holds cell c's
    // range and offset; the candidates of the 32 cells, in cell order, are then taken 32
    // at a time with every lane busy (the same pair order as a cell-by-cell walk).
    const int nx = mx[0] - mn[0] + 1, ny = mx[1] - mn[1] + 1, ncell = nx * ny * (mx[2] - mn[2] + 1);
    for (int c0 = 0; c0 < ncell; c0 += 32) {
        const int c = c0 + lane;
        int qb = 0, len = 0, shift = 0;
        float ox = 0.f, oy = 0.f, oz = 0.f;
        if (c < ncell) {
            const int i2 = mn[0] + c % nx, j2 = mn[1] + (c / nx) % ny, k2 = mn[2] + c / (nx * ny);
            const int t = cc[2] + k2, u = cc[1] + j2, v = cc[0] + i2;
            const int k3 = g.cellsN[2] > 1 ? ((t % g.cellsN[2]) + g.cellsN[2]) % g.cellsN[2] : 0;
            const int j3 = g.cellsN[1] > 1 ? ((u % g.cellsN[1]) + g.cellsN[1]) % g.cellsN[1] : 0;
            const int i3 = g.cellsN[0] > 1 ? ((v % g.cellsN[0]) + g.cellsN[0]) % g.cellsN[0] : 0;
            const int k4 = (t - k3) / g.cellsN[2], j4 = (u - j3) / g.cellsN[1], i4 = (v - i3) / g.cellsN[0];
            const int cl_loc = i3 + g.cellsN[0] * (j3 + g.cellsN[1] * k3);
            const int cl = g.cell_base + cl_loc;
            ox = g.lat32[0] * i4 + g.lat32[3] * j4 + g.lat32[6] * k4 - pa32.x;
            oy = g.lat32[1] * i4 + g.lat32[4] * j4 + g.lat32[7] * k4 - pa32.y;
            oz = g.lat32[2] * i4 + g.lat32[5] * j4 + g.lat32[8] * k4 - pa32.z;
            // cell shift in 10 bits per axis (|shift| <= img + 1 < 512) and the same-cell flag
            shift = pack_shift(i4, j4, k4) | ((cl_loc == lin) ? (1 << 30) : 0);
            const int q0 = cstart[cl];
            len = cend[cl] - q0;
            qb = q0;
        }
        int incl = len;
        for (int o = 1; o < 32; o <<= 1) {
            const int x = __shfl_up_sync(full, incl, o);
            if (lane >= o) incl += x;
        }
        const int total = __shfl_sync(full, incl, 31);
        qb -= incl - len;  // candidate f of this cell is sorted[qb + f]
        for (int f0 = 0; f0 < total; f0 += 32) {
            const int f = f0 + lane;
            // owner cell: the number of cells whose candidates all precede f
            int own = 0;
            for (int step = 16; step >= 1; step >>= 1) {
                const int x = __shfl_sync(full, incl, own + step - 1);
                if (x <= f) own += step;
            }
            own = min(own, 31);
            const int q = __shfl_sync(full, qb, own) + f;
            const int sh = __shfl_sync(full, shift, own);
            const float fox = __shfl_sync(full, ox, own), foy = __shfl_sync(full, oy, own),
                        foz = __shfl_sync(full, oz, own);
            bool keep = false;
            int b = -1, s0 = 0, s1 = 0, s2 = 0;
            double d0 = 0, d1 = 0, d2 = 0, r = 0;
            if (f < total) {
                const int i4 = (sh & 1023) - 512, j4 = ((sh >> 10) & 1023) - 512, k4 = ((sh >> 20) & 1023) - 512;
                const bool same_cell = (sh >> 30) & 1;
                b = sorted[q];
                const float4 pb = wpos[q];
                float fx = pb.x + fox, fy = pb.y + foy, fz = pb.z + foz;
                const bool self0 = (b == a && i4 == 0 && j4 == 0 && k4 == 0 && same_cell);
                const float r2 = fx * fx + fy * fy + fz * fz;
                const bool sure = r2 < sure2;
                if (!FILL && sure && !self0) keep = true;
                else if (!self0 && r2 < lim2) {
                    s0 = i4 - msa0 + ms[3 * b]; s1 = j4 - msa1 + ms[3 * b + 1]; s2 = k4 - msa2 + ms[3 * b + 2];
                    if (MIXED && sure) {
                        pair_vector_mixed(phi, plo, g, a, b, s0, s1, s2, d0, d1, d2, r);
                        keep = true;
                    } else {
                        pair_vector(pos, g.lat, a, b, s0, s1, s2, d0, d1, d2, r);
                        keep = sure || (!(d0 > cutoff || d1 > cutoff || d2 > cutoff) && r < cutoff);
                    }
                }
            }
            const unsigned m = __ballot_sync(full, keep);
            if (FILL && keep) {
                const int p = base + count + __popc(m & lt);
                nj[p] = b;
                if (CALLER_LAYOUT) {
                    ns[3 * (size_t)p] = s0;
                    ns[3 * (size_t)p + 1] = s1;
                    ns[3 * (size_t)p + 2] = s2;
                } else {
                    nd[p] = make_double4(d0, d1, d2, r);
                    ns[p] = pack_shift(s0, s1, s2);
                    ni[p] = a;
                }
                if (r < 1e-10) atomicOr(bad, 2);
            }
            count += __popc(m);
        }
    }
    if (!FILL && lane == 0) cnt[a] = count;
}

__global__ void k_reverse(long long P, const int* __restrict__ off, const int* __restrict__ nj, const int* __restrict__ ni,
                          const int* __restrict__ ns, int* __restrict__ rev, int* __restrict__ bad) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int a = ni[p], b = nj[p], s = ns[p];
    const int s0 = (s & 1023) - 512, s1 = ((s >> 10) & 1023) - 512, s2 = ((s >> 20) & 1023) - 512;
    // one search per unordered pair: the direction with a < b (a == b: the lexicographically
    // positive image shift) finds its partner and writes both entries
    if (a > b || (a == b && !(s0 > 0 || (s0 == 0 && (s1 > 0 || (s1 == 0 && s2 > 0)))))) return;
    const int want = pack_shift(-s0, -s1, -s2);
    int found = -1;
    for (int q = off[b]; q < off[b + 1]; ++q)
        if (nj[q] == a && ns[q] == want) { found = q; break; }
    rev[p] = found;
    if (found >= 0) rev[found] = (int)p;
    else atomicOr(bad, 4);
}

// rev starts at -1 (memset before k_reverse): a pair whose partner direction is missing
// (an asymmetric list) keeps -1 and sets bit 4 here
__global__ void k_rev_check(long long P, const int* __restrict__ rev, int* __restrict__ bad) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p < P && rev[p] < 0) atomicOr(bad, 4);
}

// connection_calc_dists: new displacements for an existing list (same formula as the
// fill pass, so a refreshed list equals a rebuilt one entry for entry).
template <bool MIXED>
__global__ void k_distances(long long P, const double* __restrict__ pos, const float4* __restrict__ phi,
                            const float4* __restrict__ plo, const GeomDev* __restrict__ geoms, const int* __restrict__ sid,
                            const int* __restrict__ ni, const int* __restrict__ nj, const int* __restrict__ ns,
                            double4* __restrict__ nd, int* __restrict__ bad) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p >= P) return;
    const int a = ni[p], b = nj[p], s = ns[p];
    const GeomDev& g = geoms[sid_of(sid, a)];
    double d0, d1, d2, r;
    const int s0 = (s & 1023) - 512, s1 = ((s >> 10) & 1023) - 512, s2 = ((s >> 20) & 1023) - 512;
    if (MIXED) pair_vector_mixed(phi, plo, g, a, b, s0, s1, s2, d0, d1, d2, r);
    else pair_vector(pos, g.lat, a, b, s0, s1, s2, d0, d1, d2, r);
    nd[p] = make_double4(d0, d1, d2, r);
    if (r < 1e-10) atomicOr(bad, 2);
}

__global__ void k_zero_shift(long long P, int* __restrict__ ns) {
    long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (p < P) ns[p] = pack_shift(0, 0, 0);
}

// Largest displacement since the list was built, minimum image on periodic axes
// (distance_min_image of Connection.f95:1108).  Non-negative doubles order like their
// bit patterns, so the maximum is an integer atomicMax.
__global__ void k_max_disp(int n, const double* __restrict__ pos, const double* __restrict__ ref,
                           const GeomDev* __restrict__ geoms, const int* __restrict__ sid,
                           unsigned long long* __restrict__ out) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    double dmax = 0.0;
    if (a < n) {
        const GeomDev& g = geoms[sid_of(sid, a)];
        double dp[3] = {pos[3 * a] - ref[3 * a], pos[3 * a + 1] - ref[3 * a + 1], pos[3 * a + 2] - ref[3 * a + 2]};
        double f[3];
        for (int d = 0; d < 3; ++d) {
            f[d] = g.ginv[d] * dp[0] + g.ginv[3 + d] * dp[1] + g.ginv[6 + d] * dp[2];
            if (g.pbc[d]) f[d] -= rint(f[d]);
        }
        double c2 = 0;
        for (int d = 0; d < 3; ++d) {
            double x = g.lat[d] * f[0] + g.lat[3 + d] * f[1] + g.lat[6 + d] * f[2];
            c2 += x * x;
        }
        dmax = sqrt(c2);
    }
    for (int o = 16; o > 0; o >>= 1) dmax = fmax(dmax, __shfl_xor_sync(0xffffffffu, dmax, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(dmax));
}

// Per-structure extent in fractional coordinates of the true lattice (calc_lat_eff):
// one block per structure.
__global__ void k_latpos_minmax(const double* __restrict__ pos, const GeomDev* __restrict__ geoms, double* __restrict__ out) {
    __shared__ double smn[3][256], smx[3][256];
    const GeomDev& g = geoms[blockIdx.x];
    double mn[3] = {1e300, 1e300, 1e300}, mx[3] = {-1e300, -1e300, -1e300};
    for (int a = g.atom_begin + threadIdx.x; a < g.atom_end; a += blockDim.x) {
        for (int d = 0; d < 3; ++d) {
            double lp = g.ginv[d] * pos[3 * a] + g.ginv[3 + d] * pos[3 * a + 1] + g.ginv[6 + d] * pos[3 * a + 2];
            mn[d] = fmin(mn[d], lp); mx[d] = fmax(mx[d], lp);
        }
    }
    for (int d = 0; d < 3; ++d) { smn[d][threadIdx.x] = mn[d]; smx[d][threadIdx.x] = mx[d]; }
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int d = 0; d < 3; ++d) {
                smn[d][threadIdx.x] = fmin(smn[d][threadIdx.x], smn[d][threadIdx.x + s]);
                smx[d][threadIdx.x] = fmax(smx[d][threadIdx.x], smx[d][threadIdx.x + s]);
            }
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int d = 0; d < 3; ++d) { out[6 * blockIdx.x + d] = smn[d][0]; out[6 * blockIdx.x + 3 + d] = smx[d][0]; }
}

__global__ void k_fill_sid(const GeomDev* __restrict__ geoms, int* __restrict__ sid) {
    const GeomDev& g = geoms[blockIdx.x];
    for (int a = g.atom_begin + threadIdx.x; a < g.atom_end; a += blockDim.x) sid[a] = blockIdx.x;
}

void inv3(const double* a, double* g) {
    auto A = [&](int r, int c) { return a[3 * c + r]; };
    double det = A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) - A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
                 A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
    double inv[3][3] = {{(A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) / det, (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) / det,
                         (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) / det},
                        {(A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2)) / det, (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) / det,
                         (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) / det},
                        {(A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0)) / det, (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) / det,
                         (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) / det}};
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) g[3 * c + r] = inv[r][c];
}

double norm3(const double* v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1]; c[1] = a[2] * b[0] - a[0] * b[2]; c[2] = a[0] * b[1] - a[1] * b[0];
}

// First half of the host set-up of connection_calc_connect: lattice, its inverse,
// boundary conditions.
int geom_begin(const double* lattice, const int* pbc, double cutoff, GeomDev& g) {
    if (!(cutoff >= 0.0)) GG_FAIL(GAPGPU_ERR_ATOMS, "calc_connect: negative cutoff radius");
    std::memset(&g, 0, sizeof g);
    std::memcpy(g.lat, lattice, sizeof g.lat);
    g.cutoff = cutoff;
    for (int d = 0; d < 3; ++d) g.pbc[d] = pbc[d] ? 1 : 0;
    inv3(lattice, g.ginv);
    for (double v : g.ginv) if (!std::isfinite(v)) GG_FAIL(GAPGPU_ERR_ATOMS, "lattice is singular");
    std::memcpy(g.lat_eff_inv, g.ginv, sizeof g.ginv);
    return GAPGPU_OK;
}

// Second half: effective lattice of clusters and mixed boundary conditions
// (calc_lat_eff, Connection.f95:740-763, from the fractional extent mm of the atoms),
// cell grid (divide_cell), image ranges (fit_box_in_cell) and the FP32 pre-filter.
int geom_finish(GeomDev& g, int n, const double* mm) {
    const double* lattice = g.lat;
    const double cutoff = g.cutoff;
    double lat_eff[9];
    std::memcpy(lat_eff, lattice, sizeof lat_eff);
    if (mm) {
        for (int d = 0; d < 3; ++d) {
            if (g.pbc[d]) continue;
            if (mm[d] <= 0.5 || mm[3 + d] >= 0.5) {
                double ext = (mm[3 + d] - mm[d]) * 1.1;
                double nv = norm3(lattice + 3 * d);
                for (int k = 0; k < 3; ++k) lat_eff[3 * d + k] = lattice[3 * d + k] / nv * ext;
                g.lat_off[d] = mm[d] - 0.05;
            }
        }
        inv3(lat_eff, g.lat_eff_inv);
    }
    // divide_cell
    {
        const double *a = lat_eff, *b = lat_eff + 3, *cc = lat_eff + 6;
        double bc[3], ca[3], ab[3];
        cross3(b, cc, bc); cross3(cc, a, ca); cross3(a, b, ab);
        double vol = std::fabs(a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2]);
        double cut = cutoff > 0 ? cutoff : 1.0;
        g.cellsN[0] = std::max(1, (int)std::min(1e6, vol / (cut * norm3(bc))));
        g.cellsN[1] = std::max(1, (int)std::min(1e6, vol / (cut * norm3(ca))));
        g.cellsN[2] = std::max(1, (int)std::min(1e6, vol / (cut * norm3(ab))));
        // Bound the cell grid by the atom count.  The reference's search is complete
        // (every pair inside the cutoff is found: cells are at least one cutoff wide
        // and the image range covers the cutoff sphere), so coarser cells scan a
        // superset of candidates and the distance test returns the identical set.
        while ((long long)g.cellsN[0] * g.cellsN[1] * g.cellsN[2] > 4LL * n + 64) {
            int d = (g.cellsN[0] >= g.cellsN[1] && g.cellsN[0] >= g.cellsN[2]) ? 0 : (g.cellsN[1] >= g.cellsN[2] ? 1 : 2);
            g.cellsN[d] = std::max(1, g.cellsN[d] / 2);
        }
    }
    // fit_box_in_cell on the true lattice
    {
        double mx[3] = {0, 0, 0};
        for (int k = -1; k <= 1; k += 2)
            for (int j = -1; j <= 1; j += 2)
                for (int i = -1; i <= 1; i += 2) {
                    double v[3] = {i * cutoff, j * cutoff, k * cutoff};
                    for (int d = 0; d < 3; ++d)
                        mx[d] = std::max(mx[d], std::fabs(g.ginv[d] * v[0] + g.ginv[3 + d] * v[1] + g.ginv[6 + d] * v[2]));
                }
        for (int d = 0; d < 3; ++d) {
            int nn = (int)std::ceil(2.0 * mx[d]);
            g.img[d] = std::max(1, (nn + 1) / 2);
        }
        if ((long long)(2 * g.img[0] + 1) * (2 * g.img[1] + 1) * (2 * g.img[2] + 1) > 2000000LL)
            GG_FAIL(GAPGPU_ERR_ATOMS, "calc_connect: cutoff is too large for the cell (more than 2e6 periodic images)");
        if (g.img[0] > 500 || g.img[1] > 500 || g.img[2] > 500)
            GG_FAIL(GAPGPU_ERR_ATOMS, "calc_connect: cutoff is too large for the cell (more than 500 images along an axis)");
    }
    // FP32 pre-filter data: origin of the effective cell, FP32 lattice, margin
    {
        double bsize = 0;
        for (int d = 0; d < 3; ++d) {
            g.origin[d] = lat_eff[d] * g.lat_off[0] + lat_eff[3 + d] * g.lat_off[1] + lat_eff[6 + d] * g.lat_off[2];
            bsize += norm3(lat_eff + 3 * d);
        }
        for (int k = 0; k < 9; ++k) {
            g.lat32[k] = (float)lattice[k];
            g.lat_lo[k] = (float)(lattice[k] - (double)g.lat32[k]);
        }
        double margin = 1e-3 + 1e-6 * bsize + 1e-6 * cutoff;
        g.lim2 = (float)((cutoff + margin) * (cutoff + margin));
        g.sure2 = cutoff > margin ? (float)((cutoff - margin) * (cutoff - margin)) : 0.0f;
    }
    return GAPGPU_OK;
}

bool any_open(const GeomDev& g) { return !g.pbc[0] || !g.pbc[1] || !g.pbc[2]; }

}  // namespace

int DBuf::ensure(size_t bytes) {
    if (bytes <= cap && p) return GAPGPU_OK;
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
    size_t want = std::max<size_t>(bytes + bytes / 4, 256);
    GG_CUDA(cudaMalloc(&p, want));
    cap = want;
    return GAPGPU_OK;
}
void DBuf::release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
}

int build_neighbours_batch(gapgpu_context& c, int nstruct, const int* n_atoms, const double* d_pos, const double* lattices,
                           const int* pbcs, double cutoff, bool mixed) {
    cudaStream_t st = c.stream;
    if (nstruct < 1) GG_FAIL(GAPGPU_ERR_ARG, "neighbour build: no structures");
    std::vector<GeomDev>& hg = c.h_geoms;
    hg.assign(nstruct, GeomDev{});
    int n = 0, rc;
    bool open = false;
    for (int s = 0; s < nstruct; ++s) {
        if (n_atoms[s] < 0) GG_FAIL(GAPGPU_ERR_ARG, "negative atom count");
        if ((rc = geom_begin(lattices + 9 * s, pbcs + 3 * s, cutoff, hg[s]))) return rc;
        hg[s].atom_begin = n;
        n += n_atoms[s];
        hg[s].atom_end = n;
        open = open || any_open(hg[s]);
    }
    if ((rc = c.geoms.ensure(sizeof(GeomDev) * nstruct))) return rc;
    const int* sid = nullptr;
    if (nstruct > 1) {
        if ((rc = c.sid.ensure(sizeof(int) * std::max(n, 1)))) return rc;
        sid = c.sid.as<int>();
    }
    std::vector<double> mm;
    if (open || nstruct > 1) {
        GG_CUDA(cudaMemcpyAsync(c.geoms.p, hg.data(), sizeof(GeomDev) * nstruct, cudaMemcpyHostToDevice, st));
        if (nstruct > 1) {
            k_fill_sid<<<nstruct, 128, 0, st>>>(c.geoms.as<GeomDev>(), c.sid.as<int>());
            c.launches++;
        }
        if (open) {
            if ((rc = c.minmax.ensure(6 * sizeof(double) * nstruct))) return rc;
            k_latpos_minmax<<<nstruct, 256, 0, st>>>(d_pos, c.geoms.as<GeomDev>(), c.minmax.as<double>());
            c.launches++;
            mm.resize(6 * (size_t)nstruct);
            GG_CUDA(cudaMemcpyAsync(mm.data(), c.minmax.p, sizeof(double) * mm.size(), cudaMemcpyDeviceToHost, st));
        }
        GG_CUDA(cudaStreamSynchronize(st));
    }
    long long ncell = 0;
    for (int s = 0; s < nstruct; ++s) {
        if ((rc = geom_finish(hg[s], n_atoms[s], any_open(hg[s]) ? &mm[6 * (size_t)s] : nullptr))) return rc;
        hg[s].cell_base = (int)ncell;
        ncell += (long long)hg[s].cellsN[0] * hg[s].cellsN[1] * hg[s].cellsN[2];
    }
    if (ncell > (1LL << 30)) GG_FAIL(GAPGPU_ERR_ATOMS, "calc_connect: too many cells");
    GG_CUDA(cudaMemcpyAsync(c.geoms.p, hg.data(), sizeof(GeomDev) * nstruct, cudaMemcpyHostToDevice, st));
    c.n_atoms_built = n;
    c.n_pairs = 0;
    if (n == 0) return GAPGPU_OK;
    const GeomDev* dg = c.geoms.as<GeomDev>();
    if ((rc = c.cell_key.ensure(sizeof(int) * n)) || (rc = c.cell_key2.ensure(sizeof(int) * n)) ||
        (rc = c.atom_idx.ensure(sizeof(int) * n)) || (rc = c.atom_idx2.ensure(sizeof(int) * n)) ||
        (rc = c.ms.ensure(sizeof(int) * 3 * n)) || (rc = c.cell_start.ensure(sizeof(int) * ncell)) ||
        (rc = c.cell_end.ensure(sizeof(int) * ncell)) || (rc = c.nbr_cnt.ensure(sizeof(int) * (n + 1))) ||
        (rc = c.nbr_off.ensure(sizeof(int) * (n + 1))) || (rc = c.total.ensure(sizeof(int) * 4)) ||
        (rc = c.wpos.ensure(sizeof(float4) * n)) || (rc = c.phi.ensure(sizeof(float4) * n)) ||
        (rc = c.plo.ensure(sizeof(float4) * n)))
        return rc;
    c.nbr_mixed = mixed;
    int* bad = c.total.as<int>() + 2;
    GG_CUDA(cudaMemsetAsync(c.total.p, 0, sizeof(int) * 4, st));
    if (mixed) {
        k_split_pos<<<(n + 255) / 256, 256, 0, st>>>(n, d_pos, c.phi.as<float4>(), c.plo.as<float4>());
        c.launches++;
    }
    const int TB = 128, nb = (n + TB - 1) / TB;
    const int nbw = (int)(((long long)n * 32 + TB - 1) / TB);  // one warp per atom
    k_assign<<<nb, TB, 0, st>>>(n, d_pos, dg, sid, c.cell_key.as<int>(), c.atom_idx.as<int>(), c.ms.as<int>(), bad);
    // stable sort atoms by cell
    int endbit = 1;
    while ((1LL << endbit) < ncell && endbit < 31) ++endbit;
    size_t tmp = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp, c.cell_key.as<int>(), c.cell_key2.as<int>(), c.atom_idx.as<int>(),
                                    c.atom_idx2.as<int>(), n, 0, endbit, st);
    size_t tmp2 = 0;
    cub::DeviceScan::ExclusiveSum(nullptr, tmp2, c.nbr_cnt.as<int>(), c.nbr_off.as<int>(), n + 1, st);
    if ((rc = c.cub_tmp.ensure(std::max(tmp, tmp2)))) return rc;
    GG_CUDA(cub::DeviceRadixSort::SortPairs(c.cub_tmp.p, tmp, c.cell_key.as<int>(), c.cell_key2.as<int>(),
                                            c.atom_idx.as<int>(), c.atom_idx2.as<int>(), n, 0, endbit, st));
    GG_CUDA(cudaMemsetAsync(c.cell_start.p, 0, sizeof(int) * ncell, st));
    GG_CUDA(cudaMemsetAsync(c.cell_end.p, 0, sizeof(int) * ncell, st));
    k_cell_ranges<<<nb, TB, 0, st>>>(n, c.cell_key2.as<int>(), c.cell_start.as<int>(), c.cell_end.as<int>());
    k_wrapped<<<nb, TB, 0, st>>>(n, d_pos, dg, sid, c.atom_idx2.as<int>(), c.ms.as<int>(), c.wpos.as<float4>());
    k_pairs<false><<<nbw, TB, 0, st>>>(n, d_pos, c.wpos.as<float4>(), nullptr, nullptr, dg, sid, c.cell_key.as<int>(),
                                       c.ms.as<int>(), c.atom_idx2.as<int>(), c.cell_start.as<int>(), c.cell_end.as<int>(),
                                       c.nbr_cnt.as<int>(), nullptr, nullptr, nullptr, nullptr, nullptr, bad);
    GG_CUDA(cudaMemsetAsync(c.nbr_cnt.as<int>() + n, 0, sizeof(int), st));
    GG_CUDA(cub::DeviceScan::ExclusiveSum(c.cub_tmp.p, tmp2, c.nbr_cnt.as<int>(), c.nbr_off.as<int>(), n + 1, st));
    int tot = 0;
    GG_CUDA(cudaMemcpyAsync(&tot, c.nbr_off.as<int>() + n, sizeof(int), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    c.launches += 6;
    if (tot < 0) GG_FAIL(GAPGPU_ERR_ATOMS, "neighbour list larger than 2^31 entries");
    c.n_pairs = tot;
    size_t P = std::max(tot, 1);
    if ((rc = c.nbr_j.ensure(sizeof(int) * P)) || (rc = c.nbr_d.ensure(sizeof(double4) * P)) ||
        (rc = c.nbr_s.ensure(sizeof(int) * P)) || (rc = c.nbr_rev.ensure(sizeof(int) * P)) ||
        (rc = c.nbr_i.ensure(sizeof(int) * P)))
        return rc;
    if (mixed)
        k_pairs<true, false, true><<<nbw, TB, 0, st>>>(
            n, d_pos, c.wpos.as<float4>(), c.phi.as<float4>(), c.plo.as<float4>(), dg, sid, c.cell_key.as<int>(),
            c.ms.as<int>(), c.atom_idx2.as<int>(), c.cell_start.as<int>(), c.cell_end.as<int>(), nullptr,
            c.nbr_off.as<int>(), c.nbr_j.as<int>(), c.nbr_d.as<double4>(), c.nbr_s.as<int>(), c.nbr_i.as<int>(), bad);
    else
        k_pairs<true><<<nbw, TB, 0, st>>>(n, d_pos, c.wpos.as<float4>(), nullptr, nullptr, dg, sid, c.cell_key.as<int>(),
                                          c.ms.as<int>(), c.atom_idx2.as<int>(), c.cell_start.as<int>(),
                                          c.cell_end.as<int>(), nullptr, c.nbr_off.as<int>(), c.nbr_j.as<int>(),
                                          c.nbr_d.as<double4>(), c.nbr_s.as<int>(), c.nbr_i.as<int>(), bad);
    if (tot > 0) {
        GG_CUDA(cudaMemsetAsync(c.nbr_rev.p, 0xff, sizeof(int) * (size_t)tot, st));
        k_reverse<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(tot, c.nbr_off.as<int>(), c.nbr_j.as<int>(),
                                                                  c.nbr_i.as<int>(), c.nbr_s.as<int>(), c.nbr_rev.as<int>(),
                                                                  bad);
        k_rev_check<<<(unsigned)((tot + 255) / 256), 256, 0, st>>>(tot, c.nbr_rev.as<int>(), bad);
        c.launches += 2;
    }
    c.launches++;
    int flags = 0;
    GG_CUDA(cudaMemcpyAsync(&flags, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    if (flags & 1) GG_FAIL(GAPGPU_ERR_ATOMS, "atom positions contain NaN or Inf");
    if (flags & 2) GG_FAIL(GAPGPU_ERR_ATOMS, "overlapping atoms: a neighbour distance is below 1e-10 (Connection.f95:1394-1398)");
    if (flags & 4) GG_FAIL(GAPGPU_ERR_ATOMS, "internal error: neighbour list is not symmetric");
    return GAPGPU_OK;
}

int build_neighbours(gapgpu_context& c, int n, const double* d_pos, const double* lattice, const int* pbc, double cutoff,
                     const int*) {
    return build_neighbours_batch(c, 1, &n, d_pos, lattice, pbc, cutoff);
}

int refresh_distances(gapgpu_context& c, const double* d_pos) {
    const long long P = c.n_pairs;
    if (P == 0) return GAPGPU_OK;
    int* bad = c.total.as<int>() + 2;
    const int* sid = c.h_geoms.size() > 1 ? c.sid.as<int>() : nullptr;
    const unsigned nb = (unsigned)((P + 255) / 256);
    if (c.nbr_mixed) {
        const int n = c.n_atoms_built;
        k_split_pos<<<(n + 255) / 256, 256, 0, c.stream>>>(n, d_pos, c.phi.as<float4>(), c.plo.as<float4>());
        k_distances<true><<<nb, 256, 0, c.stream>>>(P, d_pos, c.phi.as<float4>(), c.plo.as<float4>(), c.geoms.as<GeomDev>(),
                                                    sid, c.nbr_i.as<int>(), c.nbr_j.as<int>(), c.nbr_s.as<int>(),
                                                    c.nbr_d.as<double4>(), bad);
        c.launches += 2;
    } else {
        k_distances<false><<<nb, 256, 0, c.stream>>>(P, d_pos, nullptr, nullptr, c.geoms.as<GeomDev>(), sid,
                                                     c.nbr_i.as<int>(), c.nbr_j.as<int>(), c.nbr_s.as<int>(),
                                                     c.nbr_d.as<double4>(), bad);
        c.launches++;
    }
    GG_CUDA(cudaGetLastError());
    return GAPGPU_OK;
}

int load_external_neighbours(gapgpu_context& c, int n, const std::vector<int>& off, const std::vector<int>& nj,
                             const double* lattice, bool mixed) {
    cudaStream_t st = c.stream;
    const long long P = nj.size();
    int rc;
    const int pbc[3] = {0, 0, 0};
    c.h_geoms.assign(1, GeomDev{});
    GeomDev& g = c.h_geoms[0];
    if ((rc = geom_begin(lattice, pbc, 0.0, g))) return rc;
    g.atom_begin = 0;
    g.atom_end = n;
    for (int k = 0; k < 9; ++k) {
        g.lat32[k] = (float)lattice[k];
        g.lat_lo[k] = (float)(lattice[k] - (double)g.lat32[k]);
    }
    const size_t PP = std::max<long long>(P, 1);
    if ((rc = c.geoms.ensure(sizeof(GeomDev))) || (rc = c.nbr_off.ensure(sizeof(int) * (n + 1))) ||
        (rc = c.nbr_j.ensure(sizeof(int) * PP)) || (rc = c.nbr_d.ensure(sizeof(double4) * PP)) ||
        (rc = c.nbr_s.ensure(sizeof(int) * PP)) || (rc = c.nbr_rev.ensure(sizeof(int) * PP)) ||
        (rc = c.nbr_i.ensure(sizeof(int) * PP)) || (rc = c.total.ensure(sizeof(int) * 4)) ||
        (rc = c.phi.ensure(sizeof(float4) * std::max(n, 1))) || (rc = c.plo.ensure(sizeof(float4) * std::max(n, 1))))
        return rc;
    std::vector<int> ni(P);
    for (int a = 0; a < n; ++a)
        for (int p = off[a]; p < off[a + 1]; ++p) ni[p] = a;
    GG_CUDA(cudaMemcpyAsync(c.geoms.p, &g, sizeof(GeomDev), cudaMemcpyHostToDevice, st));
    GG_CUDA(cudaMemcpyAsync(c.nbr_off.p, off.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st));
    GG_CUDA(cudaMemsetAsync(c.total.p, 0, sizeof(int) * 4, st));
    if (P > 0) {
        GG_CUDA(cudaMemcpyAsync(c.nbr_j.p, nj.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st));
        GG_CUDA(cudaMemcpyAsync(c.nbr_i.p, ni.data(), sizeof(int) * P, cudaMemcpyHostToDevice, st));
    }
    c.n_pairs = P;
    c.n_atoms_built = n;
    c.nbr_mixed = mixed;
    if (P > 0) {
        int* bad = c.total.as<int>() + 2;
        const unsigned nb = (unsigned)((P + 255) / 256);
        k_zero_shift<<<nb, 256, 0, st>>>(P, c.nbr_s.as<int>());
        if ((rc = refresh_distances(c, c.pos.as<double>()))) return rc;
        GG_CUDA(cudaMemsetAsync(c.nbr_rev.p, 0xff, sizeof(int) * (size_t)P, st));
        k_reverse<<<nb, 256, 0, st>>>(P, c.nbr_off.as<int>(), c.nbr_j.as<int>(), c.nbr_i.as<int>(), c.nbr_s.as<int>(),
                                       c.nbr_rev.as<int>(), bad);
        k_rev_check<<<nb, 256, 0, st>>>(P, c.nbr_rev.as<int>(), bad);
        c.launches += 3;
    }
    int flags[4] = {0, 0, 0, 0};
    GG_CUDA(cudaMemcpyAsync(flags, c.total.p, sizeof flags, cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    if (flags[2] & 2) GG_FAIL(GAPGPU_ERR_ATOMS, "quip_lammps_wrapper: two atoms of a neighbour pair overlap exactly");
    if (flags[2] & 4) GG_FAIL(GAPGPU_ERR_ARG, "neighbour list is not symmetric: give each local atom its full list");
    return GAPGPU_OK;
}

int max_displacement(gapgpu_context& c, const double* d_pos, const double* d_ref, int n, double* out) {
    int rc;
    if ((rc = c.dispmax.ensure(sizeof(unsigned long long)))) return rc;
    GG_CUDA(cudaMemsetAsync(c.dispmax.p, 0, sizeof(unsigned long long), c.stream));
    if (n > 0) {
        k_max_disp<<<(n + 255) / 256, 256, 0, c.stream>>>(n, d_pos, d_ref, c.geoms.as<GeomDev>(),
                                                         c.h_geoms.size() > 1 ? c.sid.as<int>() : nullptr,
                                                         c.dispmax.as<unsigned long long>());
        c.launches++;
    }
    unsigned long long bits = 0;
    GG_CUDA(cudaMemcpyAsync(&bits, c.dispmax.p, sizeof bits, cudaMemcpyDeviceToHost, c.stream));
    GG_CUDA(cudaStreamSynchronize(c.stream));
    std::memcpy(out, &bits, sizeof(double));
    return GAPGPU_OK;
}

}  // namespace gapgpu

// ---------------------------------------------------------------------------------
// gapgpu_neighbours_static: the same neighbour build with every piece of scratch in one
// file-scope device array instead of cudaMalloc'ed buffers.
//
// Layout of the array (byte offsets, each 256-byte aligned), for n <= MAX atoms:
//   key, key2, idx, idx2    int[MAX] each     cell key / atom index before and after the sort
//   ms                      int[3 MAX]        map_shift of each atom
//   cnt                     int[MAX + 1]      per-atom pair counts (scanned into the caller's offsets)
//   cstart, cend            int[MAX_CELLS]    atom range of each cell
//   wpos                    float4[MAX]       wrapped FP32 positions in cell order
//   minmax                  double[6]         fractional extent (non-periodic axes)
//   geom                    GeomDev           geometry record of the structure
//   flags                   int[4]            error bits of the kernels
//   cub                     bytes             temporary storage of the radix sort and the scan
namespace gapgpu {
namespace {

constexpr int STATIC_MAX_ATOMS = GAPGPU_STATIC_MAX_ATOMS;
constexpr int STATIC_MAX_CELLS = 4 * STATIC_MAX_ATOMS + 64;  // build_neighbours caps cells at 4 n + 64
constexpr size_t STATIC_CUB_BYTES = size_t(4) << 20;

constexpr size_t al256(size_t v) { return (v + 255) / 256 * 256; }
constexpr size_t SO_KEY = 0;
constexpr size_t SO_KEY2 = SO_KEY + al256(sizeof(int) * STATIC_MAX_ATOMS);
constexpr size_t SO_IDX = SO_KEY2 + al256(sizeof(int) * STATIC_MAX_ATOMS);
constexpr size_t SO_IDX2 = SO_IDX + al256(sizeof(int) * STATIC_MAX_ATOMS);
constexpr size_t SO_MS = SO_IDX2 + al256(sizeof(int) * STATIC_MAX_ATOMS);
constexpr size_t SO_CNT = SO_MS + al256(sizeof(int) * 3 * STATIC_MAX_ATOMS);
constexpr size_t SO_CSTART = SO_CNT + al256(sizeof(int) * (STATIC_MAX_ATOMS + 1));
constexpr size_t SO_CEND = SO_CSTART + al256(sizeof(int) * STATIC_MAX_CELLS);
constexpr size_t SO_WPOS = SO_CEND + al256(sizeof(int) * STATIC_MAX_CELLS);
constexpr size_t SO_MINMAX = SO_WPOS + al256(sizeof(float4) * STATIC_MAX_ATOMS);
constexpr size_t SO_GEOM = SO_MINMAX + al256(sizeof(double) * 6);
constexpr size_t SO_FLAGS = SO_GEOM + al256(sizeof(GeomDev));
constexpr size_t SO_CUB = SO_FLAGS + al256(sizeof(int) * 4);
constexpr size_t STATIC_SCRATCH_BYTES = SO_CUB + STATIC_CUB_BYTES;

// Held by every GPU that loads the library, until the process exits.
static __device__ __align__(256) unsigned char g_nbr_scratch[STATIC_SCRATCH_BYTES];

// Device address of g_nbr_scratch per device.  In host code the symbol name is only a
// host-side stand-in, so the address is looked up once per device, with that device
// current, and passed to the kernels.
std::mutex g_static_mu;
unsigned char* g_static_addr[64] = {};

int static_scratch(int dev, unsigned char** out) {
    if (dev < 0 || dev >= 64) GG_FAIL(GAPGPU_ERR_CUDA, "gapgpu_neighbours_static: device ordinal above 63");
    std::lock_guard<std::mutex> lk(g_static_mu);
    if (!g_static_addr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_nbr_scratch);
        if (e != cudaSuccess || !ptr)
            GG_FAIL(GAPGPU_ERR_CUDA, std::string("gapgpu_neighbours_static: cudaGetSymbolAddress failed: ") +
                                         cudaGetErrorString(e));
        g_static_addr[dev] = static_cast<unsigned char*>(ptr);
    }
    *out = g_static_addr[dev];
    return GAPGPU_OK;
}

}  // namespace
}  // namespace gapgpu

extern "C" int gapgpu_neighbours_static(int n, const double* d_pos, const double* lattice, const int32_t* pbc,
                                        double cutoff, int32_t* d_offsets, int32_t* d_nbr_j, int32_t* d_nbr_shift,
                                        int64_t capacity, int64_t* total, void* cuda_stream) {
    using namespace gapgpu;
    if (n <= 0 || !d_pos || !lattice || !pbc || !d_offsets || !total)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_neighbours_static: bad argument");
    if (n > STATIC_MAX_ATOMS)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_neighbours_static: " + std::to_string(n) + " atoms is above the static limit of " +
                                    std::to_string(STATIC_MAX_ATOMS) + " (use gapgpu_neighbours)");
    int dev = 0;
    GG_CUDA(cudaGetDevice(&dev));
    unsigned char* base = nullptr;
    int rc;
    if ((rc = static_scratch(dev, &base))) return rc;
    int* key = reinterpret_cast<int*>(base + SO_KEY);
    int* key2 = reinterpret_cast<int*>(base + SO_KEY2);
    int* idx = reinterpret_cast<int*>(base + SO_IDX);
    int* idx2 = reinterpret_cast<int*>(base + SO_IDX2);
    int* ms = reinterpret_cast<int*>(base + SO_MS);
    int* cnt = reinterpret_cast<int*>(base + SO_CNT);
    int* cstart = reinterpret_cast<int*>(base + SO_CSTART);
    int* cend = reinterpret_cast<int*>(base + SO_CEND);
    float4* wpos = reinterpret_cast<float4*>(base + SO_WPOS);
    double* minmax = reinterpret_cast<double*>(base + SO_MINMAX);
    int* bad = reinterpret_cast<int*>(base + SO_FLAGS);
    void* cub_tmp = base + SO_CUB;

    GeomDev* dg = reinterpret_cast<GeomDev*>(base + SO_GEOM);
    cudaStream_t st = static_cast<cudaStream_t>(cuda_stream);
    GeomDev g;
    if ((rc = geom_begin(lattice, pbc, cutoff, g))) return rc;
    g.atom_begin = 0;
    g.atom_end = n;
    double mm[6];
    if (any_open(g)) {  // fractional extent of the atoms for calc_lat_eff
        GG_CUDA(cudaMemcpyAsync(dg, &g, sizeof g, cudaMemcpyHostToDevice, st));
        k_latpos_minmax<<<1, 256, 0, st>>>(d_pos, dg, minmax);
        GG_CUDA(cudaMemcpyAsync(mm, minmax, sizeof mm, cudaMemcpyDeviceToHost, st));
        GG_CUDA(cudaStreamSynchronize(st));
    }
    if ((rc = geom_finish(g, n, any_open(g) ? mm : nullptr))) return rc;
    GG_CUDA(cudaMemcpyAsync(dg, &g, sizeof g, cudaMemcpyHostToDevice, st));
    const int ncell = g.cellsN[0] * g.cellsN[1] * g.cellsN[2];
    if (ncell > STATIC_MAX_CELLS) GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_neighbours_static: cell grid above the static limit");
    int endbit = 1;
    while ((1 << endbit) < ncell && endbit < 31) ++endbit;
    size_t t_sort = 0, t_scan = 0;
    GG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, t_sort, key, key2, idx, idx2, n, 0, endbit, st));
    GG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, t_scan, cnt, d_offsets, n + 1, st));
    if (std::max(t_sort, t_scan) > STATIC_CUB_BYTES)
        GG_FAIL(GAPGPU_ERR_ARG, "gapgpu_neighbours_static: sort workspace above the static limit");
    // The array keeps the previous call's contents: clear what the kernels accumulate into.
    GG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int) * 4, st));
    GG_CUDA(cudaMemsetAsync(cstart, 0, sizeof(int) * ncell, st));
    GG_CUDA(cudaMemsetAsync(cend, 0, sizeof(int) * ncell, st));
    GG_CUDA(cudaMemsetAsync(cnt + n, 0, sizeof(int), st));
    const int TB = 128, nb = (n + TB - 1) / TB;
    const int nbw = (int)(((long long)n * 32 + TB - 1) / TB);
    k_assign<<<nb, TB, 0, st>>>(n, d_pos, dg, nullptr, key, idx, ms, bad);
    GG_CUDA(cub::DeviceRadixSort::SortPairs(cub_tmp, t_sort, key, key2, idx, idx2, n, 0, endbit, st));
    k_cell_ranges<<<nb, TB, 0, st>>>(n, key2, cstart, cend);
    k_wrapped<<<nb, TB, 0, st>>>(n, d_pos, dg, nullptr, idx2, ms, wpos);
    k_pairs<false><<<nbw, TB, 0, st>>>(n, d_pos, wpos, nullptr, nullptr, dg, nullptr, key, ms, idx2, cstart, cend, cnt,
                                       nullptr, nullptr, nullptr, nullptr, nullptr, bad);
    GG_CUDA(cub::DeviceScan::ExclusiveSum(cub_tmp, t_scan, cnt, d_offsets, n + 1, st));
    int tot = 0;
    GG_CUDA(cudaMemcpyAsync(&tot, d_offsets + n, sizeof(int), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    if (tot < 0) GG_FAIL(GAPGPU_ERR_ATOMS, "neighbour list larger than 2^31 entries");
    *total = tot;
    if (tot > 0 && capacity >= tot && d_nbr_j && d_nbr_shift)
        k_pairs<true, true><<<nbw, TB, 0, st>>>(n, d_pos, wpos, nullptr, nullptr, dg, nullptr, key, ms, idx2, cstart, cend,
                                                nullptr, d_offsets, d_nbr_j, nullptr, d_nbr_shift, nullptr, bad);
    int flags = 0;
    GG_CUDA(cudaMemcpyAsync(&flags, bad, sizeof(int), cudaMemcpyDeviceToHost, st));
    GG_CUDA(cudaStreamSynchronize(st));
    GG_CUDA(cudaGetLastError());
    if (flags & 1) GG_FAIL(GAPGPU_ERR_ATOMS, "atom positions contain NaN or Inf");
    if (flags & 2) GG_FAIL(GAPGPU_ERR_ATOMS, "overlapping atoms: a neighbour distance is below 1e-10 (Connection.f95:1394-1398)");
    return GAPGPU_OK;
}
