// gap_oracle.cpp -- FP64 CPU restatement of QUIP's GAP energy/force/virial path.
//
// TEST INFRASTRUCTURE ONLY.  This file is the parity oracle for the GPU library:
// it is called by tests/, by __graft_entry__.smoke() and by the cpu_baseline /
// `--impl reference` legs of bench.py, always as the expected result of a comparison or
// as the reported CPU baseline, never as part of the product path.
//
// Parity pins (checked by tests/test_oracle_golden.py against the reference's own
// fixtures, copied into tests/golden/ by tests/golden/make_golden.py):
//   * tests/Si.soap.cur_points.json: 100 SOAP vectors (l_max=n_max=8, rc=4) -> 7.8e-16
//   * tests/test_descriptor.py:80-190: SOAP gradients of a C2H cell       -> 1e-9
//   * tests/test_gappot.py + gap_sample.xyz + GAP.xml: distance_2b E and F
//   * tests/test_potential_cell.py: energies in cells smaller than the cutoff
//
// What is restated, and from where:
//   neighbours  -- src/libAtoms/Connection.f95: connection_calc_connect :1035-1310,
//                  test_form_bond :448-526, add_bond :585-634, partition_atoms :1519-1587,
//                  cell_of_pos :1589-1621, divide_cell :1674-1691, fit_box_in_cell
//                  :2204-2237, get_min_max_images :1448-1513, calc_lat_eff :740-763,
//                  neighbour iteration order connection_neighbour :2011-2138
//                  (neighbour2 entries first, then neighbour1).
//   SOAP        -- GAP descriptors_module (absent from the reference checkout; libAtoms/GAP
//                  submodule, .gitmodules:9-11).  Restated from the published SOAP
//                  construction (Bartok, Kondor, Csanyi, PRB 87, 184115 (2013)) with the
//                  GAP conventions recovered from the fixtures above: Gaussian radial
//                  basis on the grid r_b = b*(rc + sigma*sqrt(2*eps*ln10))/n_max,
//                  b = 0..n_max-1, collocated neighbour densities, transform
//                  T = K^-1 L (K_ab = exp(-alpha (r_a-r_b)^2), S = L L^T the r^2 overlap),
//                  power spectrum rows (ia, jb<=ia, l) scaled by sqrt(2) off the
//                  diagonal and 1/sqrt(2l+1), unit normalisation, trailing
//                  covariance_sigma0 component.
//   distance_2b -- GAP descriptors_module (absent); one descriptor per directed pair
//                  (fixture tests/test_gappot.py pins both directions and fc(r)).
//   gp_predict  -- GAP gp_predict_module (absent): ard_se and dot_product covariances,
//                  k_s scaled by delta^2 and by the sparse point's sparseCutoff.
//   assembly    -- src/Potentials/IPModel_GAP.f95:233-605 (local energy split over ci,
//                  f_gp = gradPredict.grad_data*fc + e*grad_fc, F(j) -= f_gp,
//                  virial(j) -= (pos_n - pos_centre) (x) f_gp, e0, E_scale).
//   variance    -- GAP gpCoordinates_initialise_variance_estimate / gp_predict's variance
//                  (absent submodule; set up at IPModel_GAP.f95:185-187 from the init arg
//                  gap_variance_regularisation, accumulated at :464-488).  Restated from the
//                  published sparse-GP predictive variance sigma^2(x) = k(x,x) - k^T C^-1 k
//                  with C = K_MM + lambda I (lambda = gap_variance_regularisation), k_s =
//                  k(x, x_s) the covariance without alpha or sparseCutoff; its gradient is
//                  grad k(x,x) - 2 (grad k)^T C^-1 k.  No fixture pins it (parity unpinned);
//                  the tests check its gradient against finite differences.
//
// Build: oracle/Makefile -> oracle/_build/liboracle.so (g++ -O2 -ffp-contract=off -fopenmp).

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include <algorithm>
#include <memory>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

// ---------------------------------------------------------------- dual numbers
// Value plus gradient with respect to the three Cartesian components of a
// neighbour's displacement vector.  Used so that SOAP gradients are exact
// analytic derivatives of the same arithmetic that produces the values.
struct D3 {
    double v, d[3];
    D3() : v(0), d{0, 0, 0} {}
    D3(double x) : v(x), d{0, 0, 0} {}
};
inline D3 operator+(const D3& a, const D3& b) { D3 r; r.v = a.v + b.v; for (int k = 0; k < 3; ++k) r.d[k] = a.d[k] + b.d[k]; return r; }
inline D3 operator-(const D3& a, const D3& b) { D3 r; r.v = a.v - b.v; for (int k = 0; k < 3; ++k) r.d[k] = a.d[k] - b.d[k]; return r; }
inline D3 operator-(const D3& a) { D3 r; r.v = -a.v; for (int k = 0; k < 3; ++k) r.d[k] = -a.d[k]; return r; }
inline D3 operator*(const D3& a, const D3& b) { D3 r; r.v = a.v * b.v; for (int k = 0; k < 3; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k]; return r; }
inline D3 operator*(double s, const D3& a) { D3 r; r.v = s * a.v; for (int k = 0; k < 3; ++k) r.d[k] = s * a.d[k]; return r; }
inline D3 operator/(const D3& a, const D3& b) {
    D3 r; r.v = a.v / b.v;
    for (int k = 0; k < 3; ++k) r.d[k] = (a.d[k] * b.v - a.v * b.d[k]) / (b.v * b.v);
    return r;
}
inline D3 dexp(const D3& a) { D3 r; r.v = std::exp(a.v); for (int k = 0; k < 3; ++k) r.d[k] = r.v * a.d[k]; return r; }
inline D3 dsqrt(const D3& a) { D3 r; r.v = std::sqrt(a.v); for (int k = 0; k < 3; ++k) r.d[k] = a.d[k] / (2.0 * r.v); return r; }
inline D3 dcos(const D3& a) { D3 r; r.v = std::cos(a.v); double s = -std::sin(a.v); for (int k = 0; k < 3; ++k) r.d[k] = s * a.d[k]; return r; }

// ---------------------------------------------------------------- 3x3 helpers
// Lattice is column-major: lat[3*c + k] = component k of cell vector c
// (Fortran at%lattice(k, c)).
void inv3(const double* a, double* g) {
    // a, g column-major 3x3
    auto A = [&](int r, int c) { return a[3 * c + r]; };
    double det = A(0, 0) * (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) - A(0, 1) * (A(1, 0) * A(2, 2) - A(1, 2) * A(2, 0)) +
                 A(0, 2) * (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0));
    double inv[3][3];
    inv[0][0] = (A(1, 1) * A(2, 2) - A(1, 2) * A(2, 1)) / det;
    inv[0][1] = (A(0, 2) * A(2, 1) - A(0, 1) * A(2, 2)) / det;
    inv[0][2] = (A(0, 1) * A(1, 2) - A(0, 2) * A(1, 1)) / det;
    inv[1][0] = (A(1, 2) * A(2, 0) - A(1, 0) * A(2, 2)) / det;
    inv[1][1] = (A(0, 0) * A(2, 2) - A(0, 2) * A(2, 0)) / det;
    inv[1][2] = (A(0, 2) * A(1, 0) - A(0, 0) * A(1, 2)) / det;
    inv[2][0] = (A(1, 0) * A(2, 1) - A(1, 1) * A(2, 0)) / det;
    inv[2][1] = (A(0, 1) * A(2, 0) - A(0, 0) * A(2, 1)) / det;
    inv[2][2] = (A(0, 0) * A(1, 1) - A(0, 1) * A(1, 0)) / det;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) g[3 * c + r] = inv[r][c];
}
void matvec3(const double* m, const double* x, double* y) {  // y = m x, m column-major
    for (int r = 0; r < 3; ++r) y[r] = m[r] * x[0] + m[3 + r] * x[1] + m[6 + r] * x[2];
}
void cross3(const double* a, const double* b, double* c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}
double norm3(const double* a) { return std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]); }

// ---------------------------------------------------------------- neighbour list
struct Bond { int j; int s[3]; double d; };
struct Ref { int i; int idx; };

struct NeighbourList {
    // per-atom flattened list in QUIP iteration order
    std::vector<int> off, j, shift;
    std::vector<double> diff, r;
};

// connection_calc_connect (Connection.f95:1035-1310) without skin handling:
// cell partition, image loops and the atom1<=atom2 half list, then flattened
// per atom as neighbour2 entries followed by neighbour1 entries
// (connection_neighbour, Connection.f95:2011-2138).
int build_neighbours(int n, const double* pos, const double* lat, const int* pbc, double cutoff, NeighbourList& out) {
    out.off.assign(n + 1, 0);
    out.j.clear(); out.shift.clear(); out.diff.clear(); out.r.clear();
    if (cutoff < 0.0) return -1;
    if (n == 0 || cutoff == 0.0) return 0;
    double g[9];
    inv3(lat, g);
    // calc_lat_eff (Connection.f95:740-763)
    double lat_eff[9], lat_off[3] = {0, 0, 0};
    std::memcpy(lat_eff, lat, sizeof lat_eff);
    bool any_np = !pbc[0] || !pbc[1] || !pbc[2];
    if (any_np) {
        std::vector<double> lp(3 * (size_t)n);
        for (int a = 0; a < n; ++a) matvec3(g, pos + 3 * a, &lp[3 * a]);
        for (int d = 0; d < 3; ++d) {
            if (pbc[d]) continue;
            double mn = 1e300, mx = -1e300;
            for (int a = 0; a < n; ++a) { mn = std::min(mn, lp[3 * a + d]); mx = std::max(mx, lp[3 * a + d]); }
            if (mn <= 0.5 || mx >= 0.5) {
                double ext = (mx - mn) * 1.1;
                double nv = norm3(lat + 3 * d);
                for (int k = 0; k < 3; ++k) lat_eff[3 * d + k] = lat[3 * d + k] / nv * ext;
                lat_off[d] = mn - 0.05;
            }
        }
    }
    double lat_eff_inv[9];
    inv3(lat_eff, lat_eff_inv);
    // divide_cell (Connection.f95:1674-1691)
    int cellsN[3];
    {
        const double *a = lat_eff, *b = lat_eff + 3, *c = lat_eff + 6;
        double bc[3], ca[3], ab[3];
        cross3(b, c, bc); cross3(c, a, ca); cross3(a, b, ab);
        double vol = std::fabs(a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2]);
        cellsN[0] = std::max(1, (int)(vol / (cutoff * norm3(bc))));
        cellsN[1] = std::max(1, (int)(vol / (cutoff * norm3(ca))));
        cellsN[2] = std::max(1, (int)(vol / (cutoff * norm3(ab))));
    }
    // fit_box_in_cell (Connection.f95:2204-2237) on the true lattice
    int img[3];
    {
        double mx[3] = {0, 0, 0};
        for (int k = -1; k <= 1; k += 2)
            for (int jj = -1; jj <= 1; jj += 2)
                for (int ii = -1; ii <= 1; ii += 2) {
                    double v[3] = {ii * cutoff, jj * cutoff, k * cutoff}, lc[3];
                    matvec3(g, v, lc);
                    for (int d = 0; d < 3; ++d) mx[d] = std::max(mx[d], std::fabs(lc[d]));
                }
        for (int d = 0; d < 3; ++d) {
            int nn = (int)std::ceil(2.0 * mx[d]);
            img[d] = std::max(1, (nn + 1) / 2);
        }
    }
    // partition_atoms (Connection.f95:1519-1587): linked lists, head insertion
    int ncell = cellsN[0] * cellsN[1] * cellsN[2];
    std::vector<int> head(ncell, -1), next(n, -1), ms(3 * (size_t)n), cidx(3 * (size_t)n);
    for (int a = 0; a < n; ++a) {
        double lp[3];
        matvec3(lat_eff_inv, pos + 3 * a, lp);
        for (int d = 0; d < 3; ++d) lp[d] -= lat_off[d];
        int c3[3];
        for (int d = 0; d < 3; ++d) {
            int m = pbc[d] ? -(int)std::floor(lp[d] + 0.5) : 0;
            ms[3 * a + d] = m;
            double t = lp[d] + m;
            int ci = (int)std::floor((double)cellsN[d] * (t + 0.5)) + 1;  // cell_of_pos
            if (ci < 1) ci = 1; else if (ci > cellsN[d]) ci = cellsN[d];
            c3[d] = ci;
            cidx[3 * a + d] = ci;
        }
        int lin = (c3[0] - 1) + cellsN[0] * ((c3[1] - 1) + cellsN[1] * (c3[2] - 1));
        next[a] = head[lin];
        head[lin] = a;
    }
    std::vector<std::vector<Bond>> n1(n);
    std::vector<std::vector<Ref>> n2(n);
    auto cell_at = [&](int i, int j, int k) { return head[(i - 1) + cellsN[0] * ((j - 1) + cellsN[1] * (k - 1))]; };
    for (int k = 1; k <= cellsN[2]; ++k)
        for (int j = 1; j <= cellsN[1]; ++j)
            for (int i = 1; i <= cellsN[0]; ++i) {
                int cc[3] = {i, j, k}, mn[3], mx[3];
                for (int d = 0; d < 3; ++d) {  // get_min_max_images (Connection.f95:1448-1513)
                    if (pbc[d]) { mn[d] = -img[d]; mx[d] = img[d]; }
                    else {
                        mn[d] = (img[d] < cc[d]) ? -img[d] : -cc[d] + 1;
                        mx[d] = (img[d] < cellsN[d] - cc[d]) ? img[d] : cellsN[d] - cc[d];
                    }
                }
                for (int a1 = cell_at(i, j, k); a1 >= 0; a1 = next[a1]) {
                    for (int k2 = mn[2]; k2 <= mx[2]; ++k2) {
                        int k3 = 1, k4;
                        if (cellsN[2] > 1) k3 = ((k + k2 - 1 + cellsN[2]) % cellsN[2] + cellsN[2]) % cellsN[2] + 1;
                        k4 = (k + k2 - k3) / cellsN[2];
                        for (int j2 = mn[1]; j2 <= mx[1]; ++j2) {
                            int j3 = 1, j4;
                            if (cellsN[1] > 1) j3 = ((j + j2 - 1 + cellsN[1]) % cellsN[1] + cellsN[1]) % cellsN[1] + 1;
                            j4 = (j + j2 - j3) / cellsN[1];
                            for (int i2 = mn[0]; i2 <= mx[0]; ++i2) {
                                int i3 = 1, i4;
                                if (cellsN[0] > 1) i3 = ((i + i2 - 1 + cellsN[0]) % cellsN[0] + cellsN[0]) % cellsN[0] + 1;
                                i4 = (i + i2 - i3) / cellsN[0];
                                for (int a2 = cell_at(i3, j3, k3); a2 >= 0; a2 = next[a2]) {
                                    if (a1 > a2) continue;
                                    if (a1 == a2 && i4 == 0 && j4 == 0 && k4 == 0 && i == i3 && j == j3 && k == k3) continue;
                                    int s[3] = {i4 - ms[3 * a1] + ms[3 * a2], j4 - ms[3 * a1 + 1] + ms[3 * a2 + 1],
                                                k4 - ms[3 * a1 + 2] + ms[3 * a2 + 2]};
                                    // test_form_bond (Connection.f95:448-526)
                                    double dd[3];
                                    for (int q = 0; q < 3; ++q) dd[q] = pos[3 * a2 + q] - pos[3 * a1 + q];
                                    for (int m = 0; m < 3; ++m)
                                        for (int q = 0; q < 3; ++q) dd[q] += lat[3 * m + q] * s[m];
                                    bool far = false;
                                    for (int m = 0; m < 3; ++m) if (dd[m] > cutoff) far = true;
                                    if (far) continue;
                                    double dist = std::sqrt(dd[0] * dd[0] + dd[1] * dd[1] + dd[2] * dd[2]);
                                    if (dist < cutoff) {  // add_bond (Connection.f95:585-634)
                                        Bond b; b.j = a2; b.s[0] = s[0]; b.s[1] = s[1]; b.s[2] = s[2]; b.d = dist;
                                        n1[a1].push_back(b);
                                        if (a1 != a2) n2[a2].push_back(Ref{a1, (int)n1[a1].size() - 1});
                                    }
                                }
                            }
                        }
                    }
                }
            }
    // flatten
    for (int a = 0; a < n; ++a) {
        out.off[a] = (int)out.j.size();
        auto emit = [&](int jj, const int* s, double dist) {
            out.j.push_back(jj);
            double df[3];
            for (int q = 0; q < 3; ++q) df[q] = pos[3 * jj + q] - pos[3 * a + q];
            for (int m = 0; m < 3; ++m)
                for (int q = 0; q < 3; ++q) df[q] += lat[3 * m + q] * s[m];
            for (int q = 0; q < 3; ++q) { out.shift.push_back(s[q]); out.diff.push_back(df[q]); }
            out.r.push_back(dist);
        };
        for (const Ref& rf : n2[a]) {
            const Bond& b = n1[rf.i][rf.idx];
            int s[3] = {-b.s[0], -b.s[1], -b.s[2]};
            emit(rf.i, s, b.d);
        }
        for (const Bond& b : n1[a]) emit(b.j, b.s, b.d);
    }
    out.off[n] = (int)out.j.size();
    return 0;
}

// coordination_function / its derivative: fc(r) = 1 below rc-w,
// 0.5 (cos(pi (r - rc + w)/w) + 1) in the transition, 0 above rc.
double fcut(double r, double rc, double w) {
    if (r > rc) return 0.0;
    if (r > rc - w) return 0.5 * (std::cos(M_PI * (r - rc + w) / w) + 1.0);
    return 1.0;
}
double dfcut(double r, double rc, double w) {
    if (r > rc || r <= rc - w) return 0.0;
    return -0.5 * M_PI * std::sin(M_PI * (r - rc + w) / w) / w;
}

// ---------------------------------------------------------------- SOAP
struct Soap {
    double rc, w, sigma, alpha, cw, sigma0, bee;
    int l_max, n_max, n_species, n_Z;
    std::vector<int> species_Z, Z;
    bool normalise, diagonal_radial, central_all, two_l;
    std::vector<double> rb, T;  // T[a*n_max + n]
    int dim() const {
        int N = n_max * n_species;
        int P = diagonal_radial ? N : N * (N + 1) / 2;
        if (diagonal_radial) P = n_species * (n_species + 1) / 2 * n_max;  // a == b only
        return P * (l_max + 1) + 1;
    }
};

double overlap_gauss(double a, double b, double al) {
    return std::exp(-al * (a * a + b * b)) * std::sqrt(2.0) * std::pow(al, 1.5) * (a + b) +
           al * std::exp(-0.5 * al * (a - b) * (a - b)) * std::sqrt(M_PI) * (1.0 + al * (a + b) * (a + b)) *
               (1.0 + std::erf(std::sqrt(al / 2.0) * (a + b)));
}

void soap_setup(Soap& s) {
    int n = s.n_max;
    s.alpha = 0.5 / (s.sigma * s.sigma);
    double step = (s.rc + s.sigma * std::sqrt(2.0 * s.bee * std::log(10.0))) / n;
    s.rb.resize(n);
    for (int b = 0; b < n; ++b) s.rb[b] = step * b;
    std::vector<double> S(n * n), K(n * n), L(n * n, 0.0);
    for (int a = 0; a < n; ++a)
        for (int b = 0; b < n; ++b) {
            S[a * n + b] = overlap_gauss(s.rb[a], s.rb[b], s.alpha);
            K[a * n + b] = std::exp(-s.alpha * (s.rb[a] - s.rb[b]) * (s.rb[a] - s.rb[b]));
        }
    // Cholesky S = L L^T
    for (int j = 0; j < n; ++j) {
        double d = S[j * n + j];
        for (int k = 0; k < j; ++k) d -= L[j * n + k] * L[j * n + k];
        L[j * n + j] = std::sqrt(d);
        for (int i = j + 1; i < n; ++i) {
            double v = S[i * n + j];
            for (int k = 0; k < j; ++k) v -= L[i * n + k] * L[j * n + k];
            L[i * n + j] = v / L[j * n + j];
        }
    }
    // T = K^-1 L via Gaussian elimination with partial pivoting
    std::vector<double> A = K, B = L;
    for (int c = 0; c < n; ++c) {
        int p = c;
        for (int r = c + 1; r < n; ++r) if (std::fabs(A[r * n + c]) > std::fabs(A[p * n + c])) p = r;
        if (p != c) for (int k = 0; k < n; ++k) { std::swap(A[c * n + k], A[p * n + k]); std::swap(B[c * n + k], B[p * n + k]); }
        for (int r = 0; r < n; ++r) {
            if (r == c) continue;
            double f = A[r * n + c] / A[c * n + c];
            if (f == 0.0) continue;
            for (int k = 0; k < n; ++k) { A[r * n + k] -= f * A[c * n + k]; B[r * n + k] -= f * B[c * n + k]; }
        }
    }
    s.T.assign(n * n, 0.0);
    for (int r = 0; r < n; ++r)
        for (int k = 0; k < n; ++k) s.T[r * n + k] = B[r * n + k] / A[r * n + r];
}

// exp(-alpha(r^2+rb^2)) i_l(2 alpha r rb), l = 0..l_max, as upward recurrence in
// terms of exp(-alpha (r -+ rb)^2).
template <class R>
void radial_collocation(const R& r, double rb, double alpha, int l_max, R* out) {
    double x0 = 2.0 * alpha * rb;
    if (rb == 0.0) {
        out[0] = dexp(-alpha * (r * r));
        for (int l = 1; l <= l_max; ++l) out[l] = R(0.0);
        return;
    }
    R x = x0 * r;
    R em = dexp(-alpha * ((r - R(rb)) * (r - R(rb))));
    R ep = dexp(-alpha * ((r + R(rb)) * (r + R(rb))));
    out[0] = 0.5 * (em - ep) / x;
    if (l_max >= 1) out[1] = 0.5 * (em + ep) / x - 0.5 * (em - ep) / (x * x);
    for (int l = 2; l <= l_max; ++l) out[l] = out[l - 2] - (double)(2 * l - 1) * out[l - 1] / x;
}

// Real orthonormal spherical harmonics Y_lm(d/|d|), index l*l + l + m.
// Y_lm = N_lm Q_l^|m|(z/r) * {Re,Im}[(x+iy)^|m|] / r^|m| (sqrt2 for m != 0),
// Q the associated Legendre function divided by (1-t^2)^(m/2).
template <class R>
void real_ylm(const R& x, const R& y, const R& z, const R& r, int l_max, R* Y) {
    R t = z / r;
    R xr = x / r, yr = y / r;
    int L = l_max + 1;
    std::vector<R> cm(L), sm(L);  // Re/Im (x+iy)^m / r^m
    cm[0] = R(1.0); sm[0] = R(0.0);
    for (int m = 1; m < L; ++m) {
        cm[m] = cm[m - 1] * xr - sm[m - 1] * yr;
        sm[m] = sm[m - 1] * xr + cm[m - 1] * yr;
    }
    std::vector<R> Q(L * L);
    auto q = [&](int l, int m) -> R& { return Q[l * L + m]; };
    for (int m = 0; m < L; ++m) {
        double dfact = 1.0;
        for (int k = 1; k <= 2 * m - 1; k += 2) dfact *= k;
        q(m, m) = R(dfact);
        if (m + 1 < L) q(m + 1, m) = (double)(2 * m + 1) * t * q(m, m);
        for (int l = m + 2; l < L; ++l)
            q(l, m) = ((double)(2 * l - 1) * t * q(l - 1, m) - (double)(l + m - 1) * q(l - 2, m)) * R(1.0 / (l - m));
    }
    for (int l = 0; l < L; ++l)
        for (int m = 0; m <= l; ++m) {
            double lf = 1.0;  // (l-m)!/(l+m)!
            for (int k = l - m + 1; k <= l + m; ++k) lf /= k;
            double N = std::sqrt((2 * l + 1) / (4.0 * M_PI) * lf);
            if (m == 0) Y[l * l + l] = N * q(l, 0);
            else {
                Y[l * l + l + m] = (std::sqrt(2.0) * N) * (q(l, m) * cm[m]);
                Y[l * l + l - m] = (std::sqrt(2.0) * N) * (q(l, m) * sm[m]);
            }
        }
}

int species_channel(const Soap& s, int Z) {
    for (int k = 0; k < s.n_species; ++k)
        if (s.species_Z[k] == Z || s.species_Z[k] == 0) return k;
    return -1;
}
bool is_centre(const Soap& s, int Z) {
    for (int k = 0; k < s.n_Z; ++k)
        if (s.Z[k] == Z || s.Z[k] == 0) return true;
    return false;
}

// One SOAP descriptor instance: value q (dim) and, if grad != nullptr, the
// gradient grad[(n*3 + k)*dim + d] for entry n of `ii` (0 = centre, then the
// neighbours within the cutoff in list order).  Returns the number of entries.
int soap_instance(const Soap& s, int i, const NeighbourList& nl, const int* Z, const double* pos, std::vector<double>& q,
                  std::vector<double>* grad, std::vector<int>* ii, std::vector<double>* ipos) {
    const int nm = s.n_max, L = s.l_max + 1, L2 = L * L, NS = s.n_species;
    const int dim = s.dim();
    // coefficients c[(sp*nm + n)*L2 + lm]
    std::vector<double> c((size_t)NS * nm * L2, 0.0);
    std::vector<int> nb;  // list positions within cutoff
    std::vector<int> nb_sp;
    std::vector<D3> dc;  // per neighbour: nm*L2 derivatives
    for (int p = nl.off[i]; p < nl.off[i + 1]; ++p) {
        if (nl.r[p] >= s.rc) continue;
        int sp = species_channel(s, Z[nl.j[p]]);
        if (sp < 0) continue;
        nb.push_back(p); nb_sp.push_back(sp);
    }
    const int nn = (int)nb.size();
    if (grad) dc.assign((size_t)nn * nm * L2, D3());
    std::vector<D3> Y(L2), rad((size_t)nm * L);
    for (int k = 0; k < nn; ++k) {
        int p = nb[k], sp = nb_sp[k];
        D3 x(nl.diff[3 * p]), y(nl.diff[3 * p + 1]), z(nl.diff[3 * p + 2]);
        x.d[0] = 1; y.d[1] = 1; z.d[2] = 1;
        D3 r = dsqrt(x * x + y * y + z * z);
        D3 f;
        f.v = fcut(r.v, s.rc, s.w);
        double df = dfcut(r.v, s.rc, s.w);
        for (int q3 = 0; q3 < 3; ++q3) f.d[q3] = df * r.d[q3];
        real_ylm(x, y, z, r, s.l_max, Y.data());
        for (int a = 0; a < nm; ++a) radial_collocation(r, s.rb[a], s.alpha, s.l_max, &rad[a * L]);
        for (int n = 0; n < nm; ++n)
            for (int l = 0; l < L; ++l) {
                D3 R;
                for (int a = 0; a < nm; ++a) R = R + s.T[a * nm + n] * rad[a * L + l];
                R = R * f;
                for (int m = -l; m <= l; ++m) {
                    int lm = l * l + l + m;
                    D3 v = R * Y[lm];
                    c[((size_t)sp * nm + n) * L2 + lm] += v.v;
                    if (grad) dc[((size_t)k * nm + n) * L2 + lm] = v;
                }
            }
    }
    // central atom (only l = 0)
    int zc = Z[i];
    for (int sp = 0; sp < NS; ++sp) {
        if (!(s.central_all || s.species_Z[sp] == zc || s.species_Z[sp] == 0)) continue;
        for (int n = 0; n < nm; ++n) {
            double R = 0;
            for (int a = 0; a < nm; ++a) R += s.T[a * nm + n] * std::exp(-s.alpha * s.rb[a] * s.rb[a]);
            c[((size_t)sp * nm + n) * L2 + 0] += s.cw * R * 0.5 / std::sqrt(M_PI);
        }
    }
    // power spectrum
    const int NN = NS * nm;
    std::vector<double> p(dim, 0.0);
    std::vector<int> pa, pb, pl;
    {
        int k = 0;
        for (int ia = 0; ia < NN; ++ia)
            for (int jb = 0; jb <= ia; ++jb) {
                if (s.diagonal_radial && (ia % nm) != (jb % nm)) continue;
                for (int l = 0; l < L; ++l) {
                    double v = 0;
                    for (int m = -l; m <= l; ++m) v += c[(size_t)ia * L2 + l * l + l + m] * c[(size_t)jb * L2 + l * l + l + m];
                    double fac = (ia != jb ? std::sqrt(2.0) : 1.0) * (s.two_l ? 1.0 / std::sqrt(2.0 * l + 1.0) : 1.0);
                    p[k] = v * fac;
                    pa.push_back(ia); pb.push_back(jb); pl.push_back(l);
                    ++k;
                }
            }
    }
    double nrm = 0;
    for (int d = 0; d < dim - 1; ++d) nrm += p[d] * p[d];
    nrm = std::sqrt(nrm);
    q.assign(dim, 0.0);
    for (int d = 0; d < dim - 1; ++d) q[d] = s.normalise ? p[d] / nrm : p[d];
    q[dim - 1] = s.sigma0;
    if (ii) {
        ii->assign(1, i);
        ipos->assign(pos + 3 * i, pos + 3 * i + 3);
        for (int k = 0; k < nn; ++k) {
            int pp = nb[k];
            ii->push_back(nl.j[pp]);
            for (int q3 = 0; q3 < 3; ++q3) ipos->push_back(pos[3 * i + q3] + nl.diff[3 * pp + q3]);
        }
    }
    if (!grad) return nn + 1;
    grad->assign((size_t)(nn + 1) * 3 * dim, 0.0);
    std::vector<double> dp(dim);
    for (int k = 0; k < nn; ++k) {
        int sp = nb_sp[k];
        for (int q3 = 0; q3 < 3; ++q3) {
            std::fill(dp.begin(), dp.end(), 0.0);
            for (int d = 0; d < dim - 1; ++d) {
                int ia = pa[d], jb = pb[d], l = pl[d];
                int sa = ia / nm, sb = jb / nm;
                if (sa != sp && sb != sp) continue;
                double v = 0;
                for (int m = -l; m <= l; ++m) {
                    int lm = l * l + l + m;
                    if (sa == sp) v += dc[((size_t)k * nm + ia % nm) * L2 + lm].d[q3] * c[(size_t)jb * L2 + lm];
                    if (sb == sp) v += c[(size_t)ia * L2 + lm] * dc[((size_t)k * nm + jb % nm) * L2 + lm].d[q3];
                }
                double fac = (ia != jb ? std::sqrt(2.0) : 1.0) * (s.two_l ? 1.0 / std::sqrt(2.0 * l + 1.0) : 1.0);
                dp[d] = v * fac;
            }
            double qdp = 0;
            if (s.normalise) {
                for (int d = 0; d < dim - 1; ++d) qdp += q[d] * dp[d];
            }
            double* gk = &(*grad)[((size_t)(k + 1) * 3 + q3) * dim];
            double* g0 = &(*grad)[((size_t)0 * 3 + q3) * dim];
            for (int d = 0; d < dim - 1; ++d) {
                double v = s.normalise ? (dp[d] - q[d] * qdp) / nrm : dp[d];
                gk[d] = v;
                g0[d] -= v;
            }
        }
    }
    return nn + 1;
}

// ---------------------------------------------------------------- GAP model
enum { DESC_SOAP = 1, DESC_DISTANCE_2B = 2 };
enum { COV_ARD_SE = 1, COV_DOT_PRODUCT = 2 };

struct Coordinate {
    int desc_type = 0;
    Soap soap;
    double d2_rc = 0, d2_w = 0.5;
    int d2_Z1 = 0, d2_Z2 = 0;
    int cov = 0;
    double delta = 1.0, zeta = 1.0;
    std::vector<double> theta;
    int M = 0, D = 0;
    std::vector<double> X, alpha, sc;  // X[s*D + d]
    std::vector<double> Lvar;          // Cholesky factor of K_MM + lambda I (lower, row-major), variance only
    double cutoff() const { return desc_type == DESC_SOAP ? soap.rc : d2_rc; }
};

struct Model {
    std::vector<Coordinate> coords;
    double e0[128] = {0};
    double E_scale = 1.0;
};

// gp_predict: returns e and fills gradPredict (size D) when non-null.
double gp_predict(const Coordinate& c, const double* x, double* gp) {
    double e = 0;
    if (gp) std::fill(gp, gp + c.D, 0.0);
    const double d2 = c.delta * c.delta;
    for (int s = 0; s < c.M; ++s) {
        const double* xs = &c.X[(size_t)s * c.D];
        if (c.cov == COV_DOT_PRODUCT) {
            double dot = 0;
            for (int d = 0; d < c.D; ++d) dot += x[d] * xs[d];
            double k = d2 * std::pow(dot, c.zeta) * c.sc[s];
            e += c.alpha[s] * k;
            if (gp) {
                double w = c.alpha[s] * d2 * c.zeta * std::pow(dot, c.zeta - 1.0) * c.sc[s];
                for (int d = 0; d < c.D; ++d) gp[d] += w * xs[d];
            }
        } else {
            double ss = 0;
            for (int d = 0; d < c.D; ++d) { double t = (x[d] - xs[d]) / c.theta[d]; ss += t * t; }
            double k = d2 * std::exp(-0.5 * ss) * c.sc[s];
            e += c.alpha[s] * k;
            if (gp)
                for (int d = 0; d < c.D; ++d) gp[d] += c.alpha[s] * k * (xs[d] - x[d]) / (c.theta[d] * c.theta[d]);
        }
    }
    return e;
}

// Covariance of two descriptor vectors, without alpha or sparseCutoff.
double cov_pair(const Coordinate& c, const double* x, const double* y) {
    const double d2 = c.delta * c.delta;
    if (c.cov == COV_DOT_PRODUCT) {
        double dot = 0;
        for (int d = 0; d < c.D; ++d) dot += x[d] * y[d];
        return d2 * std::pow(dot, c.zeta);
    }
    double ss = 0;
    for (int d = 0; d < c.D; ++d) {
        const double t = (x[d] - y[d]) / c.theta[d];
        ss += t * t;
    }
    return d2 * std::exp(-0.5 * ss);
}

// C = K_MM + reg I and its Cholesky factor L (C = L L^T).  Returns -1 if C is not
// positive definite.
int init_variance(Coordinate& c, double reg) {
    const int M = c.M;
    std::vector<double>& L = c.Lvar;
    L.assign((size_t)M * M, 0.0);
    for (int s = 0; s < M; ++s)
        for (int t = 0; t <= s; ++t) L[(size_t)s * M + t] = cov_pair(c, &c.X[(size_t)s * c.D], &c.X[(size_t)t * c.D]) +
                                                            (s == t ? reg : 0.0);
    for (int j = 0; j < M; ++j) {
        double dj = L[(size_t)j * M + j];
        for (int k = 0; k < j; ++k) dj -= L[(size_t)j * M + k] * L[(size_t)j * M + k];
        if (!(dj > 0)) { L.clear(); return -1; }
        dj = std::sqrt(dj);
        L[(size_t)j * M + j] = dj;
        for (int i = j + 1; i < M; ++i) {
            double v = L[(size_t)i * M + j];
            for (int k = 0; k < j; ++k) v -= L[(size_t)i * M + k] * L[(size_t)j * M + k];
            L[(size_t)i * M + j] = v / dj;
        }
    }
    return 0;
}

// sigma^2(x) = k(x,x) - k^T C^-1 k and, when grad is given, its gradient (D values).
double gp_variance(const Coordinate& c, const double* x, double* grad) {
    const int M = c.M, D = c.D;
    const std::vector<double>& L = c.Lvar;
    std::vector<double> k(M), y(M);
    for (int s = 0; s < M; ++s) k[s] = cov_pair(c, x, &c.X[(size_t)s * D]);
    for (int i = 0; i < M; ++i) {  // L z = k
        double v = k[i];
        for (int j = 0; j < i; ++j) v -= L[(size_t)i * M + j] * y[j];
        y[i] = v / L[(size_t)i * M + i];
    }
    for (int i = M - 1; i >= 0; --i) {  // L^T y = z
        double v = y[i];
        for (int j = i + 1; j < M; ++j) v -= L[(size_t)j * M + i] * y[j];
        y[i] = v / L[(size_t)i * M + i];
    }
    double var = cov_pair(c, x, x);
    for (int s = 0; s < M; ++s) var -= k[s] * y[s];
    if (grad) {
        const double d2 = c.delta * c.delta;
        std::fill(grad, grad + D, 0.0);
        if (c.cov == COV_DOT_PRODUCT) {
            double xx = 0;
            for (int d = 0; d < D; ++d) xx += x[d] * x[d];
            const double gxx = d2 * c.zeta * std::pow(xx, c.zeta - 1.0) * 2.0;
            for (int d = 0; d < D; ++d) grad[d] = gxx * x[d];
            for (int s = 0; s < M; ++s) {
                const double* xs = &c.X[(size_t)s * D];
                double dot = 0;
                for (int d = 0; d < D; ++d) dot += x[d] * xs[d];
                const double w = -2.0 * y[s] * d2 * c.zeta * std::pow(dot, c.zeta - 1.0);
                for (int d = 0; d < D; ++d) grad[d] += w * xs[d];
            }
        } else {
            for (int s = 0; s < M; ++s) {
                const double* xs = &c.X[(size_t)s * D];
                for (int d = 0; d < D; ++d) grad[d] += -2.0 * y[s] * k[s] * (xs[d] - x[d]) / (c.theta[d] * c.theta[d]);
            }
        }
    }
    return var;
}

struct Instance {
    std::vector<double> x;         // descriptor (D)
    std::vector<double> grad;      // (nent*3*D)
    std::vector<int> ii;           // atoms of the gradient entries
    std::vector<double> ipos;      // positions of the gradient entries (3*nent)
    std::vector<int> ci;           // atoms the energy is split over
    double fc = 1.0;
    std::vector<double> gfc;       // grad of covariance cutoff (3*nent)
};

// Enumerate descriptor instances in the same order as the reference descriptors.
void enumerate_instances(const Coordinate& c, int n, const int* Z, const double* pos, const NeighbourList& nl,
                         const int* mask, std::vector<std::pair<int, int>>& inst) {
    inst.clear();
    if (c.desc_type == DESC_SOAP) {
        for (int i = 0; i < n; ++i) {
            if (!is_centre(c.soap, Z[i])) continue;
            if (mask && !mask[i]) continue;
            inst.push_back({i, -1});
        }
    } else {
        for (int i = 0; i < n; ++i) {
            if (mask && !mask[i]) continue;
            for (int p = nl.off[i]; p < nl.off[i + 1]; ++p) {
                if (nl.r[p] >= c.d2_rc) continue;
                int j = nl.j[p];
                bool zi1 = c.d2_Z1 == 0 || Z[i] == c.d2_Z1, zj2 = c.d2_Z2 == 0 || Z[j] == c.d2_Z2;
                bool zi2 = c.d2_Z2 == 0 || Z[i] == c.d2_Z2, zj1 = c.d2_Z1 == 0 || Z[j] == c.d2_Z1;
                if (!((zi1 && zj2) || (zi2 && zj1))) continue;
                inst.push_back({i, p});
            }
        }
    }
}

void make_instance(const Coordinate& c, int i, int p, const int* Z, const double* pos, const NeighbourList& nl, bool do_grad,
                   Instance& I) {
    if (c.desc_type == DESC_SOAP) {
        soap_instance(c.soap, i, nl, Z, pos, I.x, do_grad ? &I.grad : nullptr, &I.ii, &I.ipos);
        I.ci.assign(1, i);
        I.fc = 1.0;
        I.gfc.assign(3 * I.ii.size(), 0.0);
    } else {
        double r = nl.r[p];
        const double* df = &nl.diff[3 * p];
        double u[3] = {df[0] / r, df[1] / r, df[2] / r};
        I.x.assign(1, r);
        I.ci = {i, nl.j[p]};
        I.fc = fcut(r, c.d2_rc, c.d2_w);
        double dfc = dfcut(r, c.d2_rc, c.d2_w);
        I.ii = {i, nl.j[p]};
        I.ipos = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], pos[3 * i] + df[0], pos[3 * i + 1] + df[1], pos[3 * i + 2] + df[2]};
        I.grad.assign(6, 0.0);
        I.gfc.assign(6, 0.0);
        for (int k = 0; k < 3; ++k) {
            I.grad[k] = -u[k];
            I.grad[3 + k] = u[k];
            I.gfc[k] = -dfc * u[k];
            I.gfc[3 + k] = dfc * u[k];
        }
    }
}

double model_cutoff(const Model& m) {
    double rc = 0;
    for (auto& c : m.coords) rc = std::max(rc, c.cutoff());
    return rc;
}

}  // namespace

// ================================================================ C ABI
extern "C" {

// Neighbour list with QUIP semantics (no minimum image).  Returns the number
// of (directed) entries; fills the arrays when capacity suffices.
long oracle_neighbours(int n, const double* pos, const double* lattice, const int* pbc, double cutoff, int* offsets, int* nbr_j,
                       int* nbr_shift, double* nbr_diff, double* nbr_r, long capacity) {
    NeighbourList nl;
    if (build_neighbours(n, pos, lattice, pbc, cutoff, nl) != 0) return -1;
    long tot = (long)nl.j.size();
    if (offsets) for (int i = 0; i <= n; ++i) offsets[i] = nl.off[i];
    if (capacity >= tot) {
        if (nbr_j) std::memcpy(nbr_j, nl.j.data(), sizeof(int) * tot);
        if (nbr_shift) std::memcpy(nbr_shift, nl.shift.data(), sizeof(int) * 3 * tot);
        if (nbr_diff) std::memcpy(nbr_diff, nl.diff.data(), sizeof(double) * 3 * tot);
        if (nbr_r) std::memcpy(nbr_r, nl.r.data(), sizeof(double) * tot);
    }
    return tot;
}

void* oracle_model_new(void) { return new Model(); }
void oracle_model_free(void* m) { delete static_cast<Model*>(m); }
void oracle_model_set_e0(void* mp, int Z, double v) {
    if (Z >= 0 && Z < 128) static_cast<Model*>(mp)->e0[Z] = v;
}
void oracle_model_set_E_scale(void* mp, double v) { static_cast<Model*>(mp)->E_scale = v; }

// fp: cutoff, transition_width, atom_sigma, central_weight, covariance_sigma0,
//     basis_error_exponent ; ip: l_max, n_max, n_species, n_Z, normalise,
//     diagonal_radial, central_reference_all_species, two_l_plus_one, then
//     species_Z[n_species], Z[n_Z]
static void fill_soap(Soap& s, const double* fp, const int* ip) {
    s.rc = fp[0]; s.w = fp[1]; s.sigma = fp[2]; s.cw = fp[3]; s.sigma0 = fp[4]; s.bee = fp[5];
    s.l_max = ip[0]; s.n_max = ip[1]; s.n_species = ip[2]; s.n_Z = ip[3];
    s.normalise = ip[4]; s.diagonal_radial = ip[5]; s.central_all = ip[6]; s.two_l = ip[7];
    s.species_Z.assign(ip + 8, ip + 8 + s.n_species);
    s.Z.assign(ip + 8 + s.n_species, ip + 8 + s.n_species + s.n_Z);
    soap_setup(s);
}

int oracle_soap_dim(const double* fp, const int* ip) {
    Soap s; fill_soap(s, fp, ip); return s.dim();
}

// cov_fp: delta, zeta, theta[D] (ard_se) ; X: M*D ; alpha, sparse_cutoff: M
int oracle_model_add_soap(void* mp, const double* fp, const int* ip, int cov, const double* cov_fp, int M, int D, const double* X,
                          const double* alpha, const double* sc) {
    Model* m = static_cast<Model*>(mp);
    Coordinate c;
    c.desc_type = DESC_SOAP;
    fill_soap(c.soap, fp, ip);
    if (c.soap.dim() != D) return -1;
    c.cov = cov; c.delta = cov_fp[0]; c.zeta = cov_fp[1];
    if (cov == COV_ARD_SE) c.theta.assign(cov_fp + 2, cov_fp + 2 + D);
    c.M = M; c.D = D;
    c.X.assign(X, X + (size_t)M * D); c.alpha.assign(alpha, alpha + M); c.sc.assign(sc, sc + M);
    m->coords.push_back(std::move(c));
    return 0;
}

int oracle_model_add_distance_2b(void* mp, double cutoff, double width, int Z1, int Z2, int cov, const double* cov_fp, int M,
                                 const double* X, const double* alpha, const double* sc) {
    Model* m = static_cast<Model*>(mp);
    Coordinate c;
    c.desc_type = DESC_DISTANCE_2B;
    c.d2_rc = cutoff; c.d2_w = width; c.d2_Z1 = Z1; c.d2_Z2 = Z2;
    c.cov = cov; c.delta = cov_fp[0]; c.zeta = cov_fp[1];
    if (cov == COV_ARD_SE) c.theta.assign(cov_fp + 2, cov_fp + 3);
    c.M = M; c.D = 1;
    c.X.assign(X, X + M); c.alpha.assign(alpha, alpha + M); c.sc.assign(sc, sc + M);
    m->coords.push_back(std::move(c));
    return 0;
}

double oracle_model_cutoff(void* mp) { return model_cutoff(*static_cast<Model*>(mp)); }

// SOAP descriptors of all centres (descriptor-level parity).  q: n_desc*dim.
// grad (optional): flattened per-entry 3*dim blocks, grad_index: (desc, atom)
// pairs.  Returns n_desc; *n_grad receives the number of gradient entries.
int oracle_soap(const double* fp, const int* ip, int n, const double* pos, const int* Z, const double* lattice, const int* pbc,
                double list_cutoff, double* q, long q_cap, double* grad, int* grad_index, long grad_cap, long* n_grad) {
    Soap s; fill_soap(s, fp, ip);
    NeighbourList nl;
    build_neighbours(n, pos, lattice, pbc, list_cutoff > 0 ? list_cutoff : s.rc, nl);
    int dim = s.dim();
    int nd = 0;
    long ng = 0;
    for (int i = 0; i < n; ++i) {
        if (!is_centre(s, Z[i])) continue;
        std::vector<double> qq, gg;
        std::vector<int> ii;
        std::vector<double> ipos;
        int ne = soap_instance(s, i, nl, Z, pos, qq, grad ? &gg : nullptr, &ii, &ipos);
        if ((long)(nd + 1) * dim <= q_cap) std::memcpy(q + (size_t)nd * dim, qq.data(), sizeof(double) * dim);
        if (grad) {
            for (int e = 0; e < ne; ++e) {
                if (ng < grad_cap) {
                    std::memcpy(grad + (size_t)ng * 3 * dim, &gg[(size_t)e * 3 * dim], sizeof(double) * 3 * dim);
                    grad_index[2 * ng] = nd;
                    grad_index[2 * ng + 1] = ii[e];
                }
                ++ng;
            }
        }
        ++nd;
    }
    if (n_grad) *n_grad = ng;
    return nd;
}

// Full GAP calculation as IPModel_GAP_Calc (IPModel_GAP.f95:233-605).
// Any output pointer may be NULL.  lattice column-major (columns = cell vectors),
// force 3*n, local_virial 9*n (column-major 3x3 per atom), mask optional.
// select/only: the calc argument only_descriptor (given, 1-based value): with more than
// one coordinate only that one is evaluated (:399-403).  epc (one value per coordinate,
// may be NULL): energy_per_coordinate, the sum of e_i * covariance_cutoff over the
// evaluated instances, before E_scale and without e0 (:462, :570).
int oracle_gap_calc_ex(void* mp, int n, const double* pos, const int* Z, const double* lattice, const int* pbc,
                       const int* mask, int select, int only, double* epc, double* energy, double* local_e, double* force,
                       double* virial, double* local_virial, int nthreads) {
    Model& m = *static_cast<Model*>(mp);
    NeighbourList nl;
    if (build_neighbours(n, pos, lattice, pbc, model_cutoff(m), nl) != 0) return -1;
    bool do_grad = force || virial || local_virial;
    std::vector<double> le(n, 0.0), f(3 * (size_t)n, 0.0), vir(9 * (size_t)n, 0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    const int ncoord = (int)m.coords.size();
    if (epc) for (int k = 0; k < ncoord; ++k) epc[k] = 0.0;
    for (int k = 0; k < ncoord; ++k) {
        const Coordinate& c = m.coords[k];
        if (select && ncoord > 1 && k + 1 != only) continue;
        std::vector<std::pair<int, int>> inst;
        enumerate_instances(c, n, Z, pos, nl, mask, inst);
        const long ni = (long)inst.size();
        double epc_k = 0.0;
#pragma omp parallel reduction(+ : epc_k)
        {
            std::vector<double> le_t(n, 0.0), f_t(3 * (size_t)n, 0.0), v_t(9 * (size_t)n, 0.0);
            std::vector<double> gp(c.D);
            Instance I;
#pragma omp for schedule(dynamic)
            for (long k = 0; k < ni; ++k) {
                make_instance(c, inst[k].first, inst[k].second, Z, pos, nl, do_grad, I);
                double e = gp_predict(c, I.x.data(), do_grad ? gp.data() : nullptr);
                epc_k += e * I.fc;
                double ec = e * I.fc / (double)I.ci.size();
                for (int a : I.ci) le_t[a] += ec;
                if (!do_grad) continue;
                int ne = (int)I.ii.size();
                for (int en = 0; en < ne; ++en) {
                    double fg[3];
                    for (int q3 = 0; q3 < 3; ++q3) {
                        const double* g = &I.grad[((size_t)en * 3 + q3) * c.D];
                        double v = 0;
                        for (int d = 0; d < c.D; ++d) v += gp[d] * g[d];
                        fg[q3] = v * I.fc + e * I.gfc[3 * en + q3];
                    }
                    int j = I.ii[en];
                    for (int q3 = 0; q3 < 3; ++q3) f_t[3 * j + q3] -= fg[q3];
                    for (int a = 0; a < 3; ++a)
                        for (int b = 0; b < 3; ++b)
                            v_t[9 * (size_t)j + 3 * b + a] -= (I.ipos[3 * en + a] - I.ipos[a]) * fg[b];
                }
            }
#pragma omp critical
            {
                for (int a = 0; a < n; ++a) le[a] += le_t[a];
                for (size_t a = 0; a < f.size(); ++a) f[a] += f_t[a];
                for (size_t a = 0; a < vir.size(); ++a) vir[a] += v_t[a];
            }
        }
        if (epc) epc[k] = epc_k;
    }
    double E = 0;
    for (int a = 0; a < n; ++a) E += le[a];
    for (int a = 0; a < n; ++a) {
        if (mask && !mask[a]) continue;
        double e0 = (Z[a] >= 0 && Z[a] < 128) ? m.e0[Z[a]] : 0.0;
        E += e0;
        le[a] += e0;
    }
    const double s = m.E_scale;
    if (energy) *energy = s * E;
    if (local_e) for (int a = 0; a < n; ++a) local_e[a] = s * le[a];
    if (force) for (size_t a = 0; a < f.size(); ++a) force[a] = s * f[a];
    if (virial) {
        for (int k = 0; k < 9; ++k) {
            double v = 0;
            for (int a = 0; a < n; ++a) v += vir[9 * (size_t)a + k];
            virial[k] = s * v;
        }
    }
    if (local_virial) for (size_t a = 0; a < vir.size(); ++a) local_virial[a] = s * vir[a];
    return 0;
}

int oracle_gap_calc(void* mp, int n, const double* pos, const int* Z, const double* lattice, const int* pbc, const int* mask,
                    double* energy, double* local_e, double* force, double* virial, double* local_virial, int nthreads) {
    return oracle_gap_calc_ex(mp, n, pos, Z, lattice, pbc, mask, 0, 0, nullptr, energy, local_e, force, virial,
                              local_virial, nthreads);
}

int oracle_model_n_coordinates(void* mp) { return (int)static_cast<Model*>(mp)->coords.size(); }

// Variance estimate set-up for every coordinate (the init arg gap_variance_regularisation,
// IPModel_GAP.f95:185-187).  Returns -1 if some K_MM + reg I is not positive definite.
int oracle_model_init_variance(void* mp, double reg) {
    for (Coordinate& c : static_cast<Model*>(mp)->coords)
        if (init_variance(c, reg) != 0) return -1;
    return 0;
}

// The calc arguments local_gap_variance / print_gap_variance (IPModel_GAP.f95:330-335,
// 464-488, 506-516): per atom local_var[a] = sum over instances with a in ci of
// sigma^2 fc^2 / |ci|, and (var_grad, 3*n, may be NULL) gap_variance_gradient(:,j) = sum
// over gradient entries n = j of grad sigma^2 . grad_data(:,:,n) fc^2 + 2 sigma^2 fc
// grad_fc(:,n).  inst_var (may be NULL, capacity inst_cap): sigma^2 of every instance, in
// instance order, coordinate after coordinate; returns the number of instances, or -1.
long oracle_gap_variance(void* mp, int n, const double* pos, const int* Z, const double* lattice, const int* pbc,
                         const int* mask, int select, int only, double* local_var, double* var_grad, double* inst_var,
                         long inst_cap, int nthreads) {
    Model& m = *static_cast<Model*>(mp);
    NeighbourList nl;
    if (build_neighbours(n, pos, lattice, pbc, model_cutoff(m), nl) != 0) return -1;
    for (const Coordinate& c : m.coords)
        if (c.Lvar.empty()) return -1;
    const bool do_grad = var_grad != nullptr;
    std::vector<double> lv(n, 0.0), g(3 * (size_t)n, 0.0);
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
    long ninst = 0;
    const int ncoord = (int)m.coords.size();
    for (int kc = 0; kc < ncoord; ++kc) {
        const Coordinate& c = m.coords[kc];
        if (select && ncoord > 1 && kc + 1 != only) continue;
        std::vector<std::pair<int, int>> inst;
        enumerate_instances(c, n, Z, pos, nl, mask, inst);
        const long ni = (long)inst.size();
        std::vector<double> var_k(ni, 0.0);
#pragma omp parallel
        {
            std::vector<double> lv_t(n, 0.0), g_t(3 * (size_t)n, 0.0), gv(c.D);
            Instance I;
#pragma omp for schedule(dynamic)
            for (long k = 0; k < ni; ++k) {
                make_instance(c, inst[k].first, inst[k].second, Z, pos, nl, do_grad, I);
                const double v = gp_variance(c, I.x.data(), do_grad ? gv.data() : nullptr);
                var_k[k] = v;
                for (int a : I.ci) lv_t[a] += v * I.fc * I.fc / (double)I.ci.size();
                if (!do_grad) continue;
                for (size_t en = 0; en < I.ii.size(); ++en) {
                    for (int q3 = 0; q3 < 3; ++q3) {
                        const double* gd = &I.grad[(en * 3 + q3) * c.D];
                        double t = 0;
                        for (int d = 0; d < c.D; ++d) t += gv[d] * gd[d];
                        g_t[3 * (size_t)I.ii[en] + q3] += t * I.fc * I.fc + 2.0 * v * I.fc * I.gfc[3 * en + q3];
                    }
                }
            }
#pragma omp critical
            {
                for (int a = 0; a < n; ++a) lv[a] += lv_t[a];
                for (size_t a = 0; a < g.size(); ++a) g[a] += g_t[a];
            }
        }
        for (long k = 0; k < ni; ++k, ++ninst)
            if (inst_var && ninst < inst_cap) inst_var[ninst] = var_k[k];
    }
    if (local_var) std::memcpy(local_var, lv.data(), sizeof(double) * n);
    if (var_grad) std::memcpy(var_grad, g.data(), sizeof(double) * 3 * n);
    return ninst;
}

}  // extern "C"
