// k_hartree.cu -- Becke-Poisson Hartree potential (MolecularGrid::calculate_hartree_potential,
// moleculargrid.cpp:336-389, and AtomicGrid::calculate_rho_lm / calculate_U_lm,
// atomicgrid.cpp:241-466).
//
// K5a rho_lm[a][lm][i] = 4 pi sum_j rho w_becke w_leb,j Y_lm(dir_j): one CTA per
//     (atom, radial shell); Y_lm of the Lebedev directions precomputed once.
// K5b radial Poisson solve per (atom, lm): the finite-difference operator
//     depends only on (nrad, l), so its solution map is built once per grid
//     (columns of the inverse from a partial-pivot LU, as the reference's dense
//     LU) and applied on the device as a matrix-vector product per (atom, lm):
//     no sequential sweeps on the slow FP64 pipe.
// K5c own-cell potential V_n(p) = sum_lm U_lm(r_i) / r Y_lm (atomicgrid.cpp:439-462).
// K5d cubic splines of U_lm over increasing r (cspline.cpp:66-142): the
//     derivatives are a fixed linear map of the ordinates (the tridiagonal
//     system depends on the abscissae only), applied per (atom, lm).  Stored
//     [atom][lm][interval][4] (interval nrad-1 holds the clamp value of the
//     last knot).
// K5e cross-atom potential: for every point and every other atom k,
//     sum_lm U^k_lm(r)/r Y_lm with Y_lm by Cartesian recursion (no atan2/acos)
//     and an O(1) spline-interval lookup from the analytic radial map
//     r = (1+x)/(1-x), x = cos(pi p/(N+1)) (moleculargrid.cpp:342-380).
//     FP64 path, or the mixed path: FP32 arithmetic per point with every
//     constant shared by many points carried as a split FP32 pair.
// Mixed path of K5a/K5c: split-FP32 products (hi*hi + hi*lo + lo*hi), FP32
//     partial sums of 16 terms added in FP64.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <tuple>
#include <vector>
#include <cub/device/device_radix_sort.cuh>
#include "dftg_internal.cuh"

namespace dftg {

// ------------------------------------------------------------------ host setup

static double fact(int n) { double r = 1.0; for (int k = 2; k <= n; ++k) r *= k; return r; }

// spherical_harmonics.cpp:28-33
static double sh_prefactor(int l, int m)
{
    const double pre = 1.0 / std::sqrt(4 * kPi);
    int am = m < 0 ? -m : m;
    return pre * (m == 0 ? 1 : std::sqrt(2.0)) * std::sqrt((double)(2 * l + 1) * fact(l - am) / fact(l + am));
}

// spherical_harmonics.cpp:81-117
static double legendre_p(int n, int m, double x)
{
    std::vector<double> v(n + 1, 0.0);
    if (m <= n) {
        v[m] = 1.0;
        double f = 1.0;
        for (int k = 0; k < m; ++k) { v[m] *= -f * std::sqrt(1.0 - x * x); f += 2.0; }
    }
    if (m + 1 <= n) v[m + 1] = x * (double)(2 * m + 1) * v[m];
    for (int j = m + 2; j <= n; ++j)
        v[j] = ((double)(2 * j - 1) * x * v[j - 1] + (double)(-j - m + 1) * v[j - 2]) / (double)(j - m);
    return v[n];
}

// Y_lm of a direction exactly as atomicgrid.cpp:282-289 evaluates it
static double ylm_host(int l, int m, double x, double y, double z)
{
    double r = std::sqrt(x * x + y * y + z * z);
    double az = std::atan2(y, x);
    double pole = std::acos(z / r);
    double a = (m == 0) ? 1.0 : (m > 0 ? std::cos((double)m * az) : std::sin(-(double)m * az));
    return sh_prefactor(l, m) * (legendre_p(l, m < 0 ? -m : m, std::cos(pole)) * a);
}

static double d2zdr2(double r, double m)
{
    double nom = m * m * (m + 3.0 * r);
    double denom = 2.0 * kPi * std::pow((m * r) / ((m + r) * (m + r)), 1.5) * std::pow(m + r, 5.0);
    return nom / denom;
}
static double dzdrsq(double r, double m) { return m / (kPi * kPi * r * (m + r) * (m + r)); }

// finite-difference operator of atomicgrid.cpp:316-389, row-major (N+2)^2
static void poisson_matrix(int N, const double *r_n, double *A)
{
    const double h = 1.0 / (double)(N + 1);
    const int S = N + 2;
    for (int t = 0; t < S * S; ++t) A[t] = 0.0;
#define M_(i, j) A[(size_t)(i) * S + (j)]
    for (int i = 0; i < S; ++i) {
        double c1 = 0.0, c2 = 0.0;
        if (i > 0 && i < N + 1) { c1 = dzdrsq(r_n[i - 1], 1.0); c2 = d2zdr2(r_n[i - 1], 1.0); }
        if (i == 0) { M_(0, 0) = 1.0; continue; }
        if (i == 1) {
            c1 /= 12.0 * h * h; c2 /= 12.0 * h;
            M_(i, 0) = 11.0 * c1 - 3.0 * c2; M_(i, 1) = -20.0 * c1 - 10.0 * c2;
            M_(i, 2) = 6.0 * c1 + 18.0 * c2; M_(i, 3) = 4.0 * c1 - 6.0 * c2;
            M_(i, 4) = -1.0 * c1 + 1.0 * c2;
            continue;
        }
        if (i == 2) {
            c1 /= 12.0 * h * h; c2 /= 60.0 * h;
            M_(i, 0) = -1.0 * c1 + 3.0 * c2; M_(i, 1) = 16.0 * c1 - 30.0 * c2;
            M_(i, 2) = -30.0 * c1 - 20.0 * c2; M_(i, 3) = 16.0 * c1 + 60.0 * c2;
            M_(i, 4) = -1.0 * c1 - 15.0 * c2; M_(i, 5) = 0.0 * c1 + 2.0 * c2;
            continue;
        }
        if (i == N - 1) {
            c1 /= 12.0 * h * h; c2 /= 60.0 * h;
            M_(i, N - 4) = 0.0 * c1 - 2.0 * c2; M_(i, N - 3) = -1.0 * c1 + 15.0 * c2;
            M_(i, N - 2) = 16.0 * c1 - 60.0 * c2; M_(i, N - 1) = -30.0 * c1 + 20.0 * c2;
            M_(i, N) = 16.0 * c1 + 30.0 * c2; M_(i, N + 1) = -1.0 * c1 - 3.0 * c2;
            continue;
        }
        if (i == N) {
            c1 /= 12.0 * h * h; c2 /= 12.0 * h;
            M_(i, N - 3) = -1.0 * c1 - 1.0 * c2; M_(i, N - 2) = 4.0 * c1 + 6.0 * c2;
            M_(i, N - 1) = 6.0 * c1 - 18.0 * c2; M_(i, N) = -20.0 * c1 + 10.0 * c2;
            M_(i, N + 1) = 11.0 * c1 + 3.0 * c2;
            continue;
        }
        if (i == N + 1) { M_(i, i) = 1.0; continue; }
        c1 /= 180.0 * h * h; c2 /= 60.0 * h;
        M_(i, i - 3) = 2.0 * c1 - 1.0 * c2; M_(i, i - 2) = -27.0 * c1 + 9.0 * c2;
        M_(i, i - 1) = 270.0 * c1 - 45.0 * c2; M_(i, i) = -490.0 * c1;
        M_(i, i + 1) = 270.0 * c1 + 45.0 * c2; M_(i, i + 2) = -27.0 * c1 - 9.0 * c2;
        M_(i, i + 3) = 2.0 * c1 + 1.0 * c2;
    }
#undef M_
}

// in-place LU with partial pivoting: multipliers below the diagonal, U above,
// piv[k] = row exchanged with k at step k
static void lu_factor(int S, double *M, int *piv);

// solve M x = b with the factors of lu_factor: row interchanges first (the rows
// were exchanged whole), then the unit-lower and upper sweeps
static void lu_apply(int S, const double *F, const int *piv, double *b)
{
    for (int k = 0; k < S; ++k)
        if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (int i = 1; i < S; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= F[(size_t)i * S + k] * b[k];
        b[i] = s;
    }
    for (int i = S - 1; i >= 0; --i) {
        double s = b[i];
        for (int j = i + 1; j < S; ++j) s -= F[(size_t)i * S + j] * b[j];
        b[i] = s / F[(size_t)i * S + i];
    }
}

// spline derivatives D of cspline.cpp:66-130 (x increasing, n >= 3)
static void spline_derivatives(int n, const double *x, const double *y, double *D)
{
    std::vector<double> A(n, 0.0), B(n, 0.0), C(n, 0.0), Y(n, 0.0);
    double h0 = x[1] - x[0], h1 = x[2] - x[1];
    double r0 = (y[1] - y[0]) / h0, r1 = (y[2] - y[1]) / h1;
    B[0] = h1 * (h0 + h1);
    C[0] = (h0 + h1) * (h0 + h1);
    Y[0] = r0 * (3 * h0 * h1 + 2 * h1 * h1) + r1 * h0 * h0;
    for (int i = 1; i < n - 1; ++i) {
        h0 = x[i] - x[i - 1];
        h1 = x[i + 1] - x[i];
        r0 = (y[i] - y[i - 1]) / h0;
        r1 = (y[i + 1] - y[i]) / h1;
        A[i] = h1;
        B[i] = 2 * (h0 + h1);
        C[i] = h0;
        Y[i] = 3 * (r0 * h1 + r1 * h0);
    }
    A[n - 1] = (h0 + h1) * (h0 + h1);
    B[n - 1] = h0 * (h0 + h1);
    Y[n - 1] = r0 * h1 * h1 + r1 * (3 * h0 * h1 + 2 * h0 * h0);
    C[0] = C[0] / B[0];
    for (int i = 1; i < n - 1; ++i) C[i] = C[i] / (B[i] - A[i] * C[i - 1]);
    Y[0] = Y[0] / B[0];
    for (int i = 1; i < n; ++i) Y[i] = (Y[i] - A[i] * Y[i - 1]) / (B[i] - A[i] * C[i - 1]);
    D[n - 1] = Y[n - 1];
    for (int i = n - 1; i > 0; --i) D[i - 1] = Y[i - 1] - C[i - 1] * D[i];
}

static void lu_factor(int S, double *M, int *piv)
{
    for (int k = 0; k < S; ++k) {
        int p = k;
        double best = std::fabs(M[(size_t)k * S + k]);
        for (int i = k + 1; i < S; ++i) {
            double v = std::fabs(M[(size_t)i * S + k]);
            if (v > best) { best = v; p = i; }
        }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < S; ++j) std::swap(M[(size_t)k * S + j], M[(size_t)p * S + j]);
        double pv = M[(size_t)k * S + k];
        for (int i = k + 1; i < S; ++i) {
            double f = M[(size_t)i * S + k] / pv;
            if (f == 0.0) continue;
            M[(size_t)i * S + k] = f;
            for (int j = k + 1; j < S; ++j) M[(size_t)i * S + j] -= f * M[(size_t)k * S + j];
        }
    }
}

static double dfact_h(int n) { double r = 1.0; for (int k = n; k > 1; k -= 2) r *= k; return r; }

// spline factor layout: inv_h, h, A, C', 1/den (each nrad) and 4 end-row constants
size_t hartree_splf_elems(int nrad) { return (size_t)5 * nrad + 4; }

static void split_f32(double v, float &hi, float &lo)
{
    hi = (float)v;
    lo = (float)(v - (double)hi);
}

// 1 / |p - atom| of every grid point, computed as in the FP64 own-cell kernel
__global__ void k_inv_radius(size_t npts, int nrad, int nang, const double *__restrict__ rn,
                             const double *__restrict__ leb, double *__restrict__ invr)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int per_atom = nrad * nang;
    const int rem = (int)(p % per_atom), i = rem / nang, j = rem % nang;
    const double ri = rn[i];
    const double px = leb[4 * j] * ri, py = leb[4 * j + 1] * ri, pz = leb[4 * j + 2] * ri;
    invr[p] = 1.0 / sqrt(px * px + py * py + pz * pz);
}

// Host tables of the Hartree step that depend only on the grid shape (radial
// points, Lebedev rule, lmax), not on the geometry: Y_lm and w Y_lm of the
// Lebedev directions, the radial Poisson maps per l, the spline derivative map
// and factorisation, the Legendre recursion coefficients and their FP32
// splits.  Built once per shape in the process and shared by every context
// (a new geometry of the same grid reuses them).
struct HartreeTables {
    std::vector<double> Y, Yw, pre, fold, Gt, Gb, Kt, rec, sx, f;
    std::vector<float> Y32, Ywt32, pre32, rec32, m32;
    std::vector<int> pairs;        // (j, antipode of j) for j < antipode; empty if a direction has none
};

// Lebedev rules are invariant under inversion: every direction j has an antipode
// -j with the same weight.  Pairs (j, antipode) with j < antipode, or nothing
// when some direction has no antipode.
static std::vector<int> antipode_pairs(int nang, const std::vector<double> &leb)
{
    std::vector<int> pairs;
    for (int j = 0; j < nang; ++j) {
        int a = -1;
        for (int k = 0; k < nang && a < 0; ++k)
            if (std::fabs(leb[4 * k] + leb[4 * j]) + std::fabs(leb[4 * k + 1] + leb[4 * j + 1]) +
                        std::fabs(leb[4 * k + 2] + leb[4 * j + 2]) < 1e-12 &&
                std::fabs(leb[4 * k + 3] - leb[4 * j + 3]) <= 1e-15 * std::fabs(leb[4 * j + 3]))
                a = k;
        if (a < 0 || a == j) return {};
        if (j < a) {
            pairs.push_back(j);
            pairs.push_back(a);
        }
    }
    return (int)pairs.size() == nang ? pairs : std::vector<int>{};
}

static std::shared_ptr<const HartreeTables> build_hartree_tables(int N, int nang, int lmax, const std::vector<double> &r_n,
                                                                 const std::vector<double> &leb)
{
    const int nlm = (lmax + 1) * (lmax + 1), S = N + 2;
    auto T = std::make_shared<HartreeTables>();
    std::vector<double> Y((size_t)nlm * nang), Yw((size_t)nlm * nang), pre(nlm), fold(nlm);
    std::vector<float> Y32(2 * (size_t)nlm * nang), Ywt32(2 * (size_t)nlm * nang);
    const size_t half = (size_t)nlm * nang;
    for (int l = 0; l <= lmax; ++l)
        for (int m = -l; m <= l; ++m) {
            const int lm = l * l + l + m, am = m < 0 ? -m : m;
            pre[lm] = sh_prefactor(l, m);
            // Y_lm = fold_lm * R_l^|m|(z) * {Re, Im}((x + i y)^|m|) with the integer recursion
            // R_l = (2l-1) z R_{l-1} - (l+m-1)(l-m-1) R_{l-2}, R_m = 1
            fold[lm] = pre[lm] * ((am & 1) ? -1.0 : 1.0) * dfact_h(2 * am - 1) / fact(l - am);
            for (int j = 0; j < nang; ++j) {
                const double y = ylm_host(l, m, leb[4 * j], leb[4 * j + 1], leb[4 * j + 2]);
                const double yw = y * leb[4 * j + 3];
                Y[(size_t)lm * nang + j] = y;
                Yw[(size_t)lm * nang + j] = yw;
                split_f32(y, Y32[(size_t)lm * nang + j], Y32[half + (size_t)lm * nang + j]);
                split_f32(yw, Ywt32[(size_t)j * nlm + lm], Ywt32[half + (size_t)j * nlm + lm]);
            }
        }
    // Radial Poisson operator per l (atomicgrid.cpp:316-425) as an explicit
    // linear map: U[i] = sum_k Gt[l][k][i] rho_lm[k] + [lm = 0] Gb[i] q_a, from
    // the columns of the inverse obtained with the partial-pivot LU factors.
    std::vector<double> A((size_t)S * S), M((size_t)S * S), e(S);
    std::vector<int> piv(S);
    std::vector<double> Gt((size_t)(lmax + 1) * N * N), Gb(N);
    poisson_matrix(N, r_n.data(), A.data());
    for (int l = 0; l <= lmax; ++l) {
        M = A;
        for (int i = 1; i < N + 1; ++i)
            M[(size_t)i * S + i] -= (double)l * (double)(l + 1) / (r_n[i - 1] * r_n[i - 1]);
        lu_factor(S, M.data(), piv.data());
        for (int k = 0; k <= N; ++k) {      // column k of the inverse
            for (int i = 0; i < S; ++i) e[i] = (i == k) ? 1.0 : 0.0;
            lu_apply(S, M.data(), piv.data(), e.data());
            for (int i = 1; i < N + 1; ++i) {
                if (k == 0) {
                    if (l == 0) Gb[i - 1] = std::sqrt(4.0 * kPi) * e[i];
                } else {
                    Gt[((size_t)l * N + (k - 1)) * N + (i - 1)] = -4.0 * kPi * r_n[k - 1] * e[i];
                }
            }
        }
    }
    // spline derivatives as a linear map of the ordinates: D = K y (cspline.cpp:66-130)
    std::vector<double> Kt((size_t)N * N);
    {
        std::vector<double> sxv(N), yv(N), D(N);
        for (int i = 0; i < N; ++i) sxv[i] = r_n[N - 1 - i];
        for (int j = 0; j < N; ++j) {
            for (int i = 0; i < N; ++i) yv[i] = (i == j) ? 1.0 : 0.0;
            spline_derivatives(N, sxv.data(), yv.data(), D.data());
            for (int i = 0; i < N; ++i) Kt[(size_t)j * N + i] = D[i];
        }
    }
    std::vector<double> rec((size_t)2 * nlm, 0.0);
    for (int l = 0; l <= lmax; ++l)
        for (int m = 0; m < l; ++m) {
            rec[2 * (l * l + l + m)] = (double)(2 * l - 1) / (double)(l - m);
            rec[2 * (l * l + l + m) + 1] = (double)(l + m - 1) / (double)(l - m);
        }
    // spline factorisation: the tridiagonal matrix of cspline.cpp:83-118 depends on x only
    std::vector<double> sx(N), f(hartree_splf_elems(N), 0.0);
    for (int i = 0; i < N; ++i) sx[i] = r_n[N - 1 - i];
    double *inv_h = f.data(), *h = inv_h + N, *Aa = h + N, *Cp = Aa + N, *inv_den = Cp + N, *k4 = inv_den + N;
    for (int i = 0; i < N - 1; ++i) { h[i] = sx[i + 1] - sx[i]; inv_h[i] = 1.0 / h[i]; }
    {
        const double h0 = h[0], h1 = h[1];
        const double B0 = h1 * (h0 + h1);
        Cp[0] = (h0 + h1) * (h0 + h1) / B0;
        inv_den[0] = 1.0 / B0;
        k4[0] = 3 * h0 * h1 + 2 * h1 * h1;   // Y_0 = r_0 k4[0] + r_1 k4[1]
        k4[1] = h0 * h0;
        for (int i = 1; i < N - 1; ++i) {
            Aa[i] = h[i];
            const double den = 2 * (h[i - 1] + h[i]) - Aa[i] * Cp[i - 1];
            Cp[i] = h[i - 1] / den;
            inv_den[i] = 1.0 / den;
        }
        const double g0 = h[N - 3], g1 = h[N - 2];
        Aa[N - 1] = (g0 + g1) * (g0 + g1);
        inv_den[N - 1] = 1.0 / (g0 * (g0 + g1) - Aa[N - 1] * Cp[N - 2]);
        k4[2] = g1 * g1;                      // Y_{n-1} = r_{n-3} k4[2] + r_{n-2} k4[3]
        k4[3] = 3 * g0 * g1 + 2 * g0 * g0;
    }
    std::vector<float> pre32(pre.begin(), pre.end()), rec32(rec.begin(), rec.end());
    // double-float copies of the fixed maps for the mixed Poisson / spline kernels:
    // [hi block][lo block] of Gt, Gb, Kt, 1/h, fold
    std::vector<float> m32;
    auto push = [&](const std::vector<double> &v, size_t n) {
        const size_t o = m32.size();
        m32.resize(o + 2 * n);
        for (size_t i = 0; i < n; ++i) split_f32(v[i], m32[o + i], m32[o + n + i]);
    };
    push(Gt, Gt.size());
    push(Gb, Gb.size());
    push(Kt, Kt.size());
    push(f, (size_t)N);                  // inv_h
    push(fold, fold.size());
    T->Y = std::move(Y); T->Yw = std::move(Yw); T->pre = std::move(pre); T->fold = std::move(fold);
    T->Gt = std::move(Gt); T->Gb = std::move(Gb); T->Kt = std::move(Kt); T->rec = std::move(rec);
    T->sx = std::move(sx); T->f = std::move(f);
    T->Y32 = std::move(Y32); T->Ywt32 = std::move(Ywt32); T->pre32 = std::move(pre32); T->rec32 = std::move(rec32);
    T->m32 = std::move(m32);
    T->pairs = antipode_pairs(nang, leb);
    return T;
}

int hartree_setup(dftg_ctx *c)
{
    const int nang = c->nang, N = c->nrad;
    DFTG_CUDA(cudaMalloc(&c->d_invr, sizeof(double) * c->npts));
    k_inv_radius<<<(unsigned)((c->npts + 255) / 256), 256, 0, c->stream>>>(c->npts, N, nang, c->d_rn, c->d_leb,
                                                                           c->d_invr);
    DFTG_LAUNCH_CHECK();
    static std::mutex mu;
    static std::map<std::tuple<int, int, int>, std::shared_ptr<const HartreeTables>> cache;
    std::shared_ptr<const HartreeTables> T;
    {
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(std::make_tuple(N, c->leb, c->lmax));
        if (it != cache.end()) T = it->second;
    }
    if (!T) {
        std::vector<double> leb((size_t)nang * 4);
        DFTG_CUDA(cudaMemcpy(leb.data(), c->d_leb, sizeof(double) * nang * 4, cudaMemcpyDeviceToHost));
        T = build_hartree_tables(N, nang, c->lmax, c->r_n, leb);
        std::lock_guard<std::mutex> lk(mu);
        cache.emplace(std::make_tuple(N, c->leb, c->lmax), T);
    }
    auto up = [&](void *dst, const void *src, size_t bytes) -> int {
        DFTG_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
        return DFTG_OK;
    };
    DFTG_CUDA(cudaMalloc(&c->d_Gt, sizeof(double) * T->Gt.size()));
    DFTG_CUDA(cudaMalloc(&c->d_Gb, sizeof(double) * T->Gb.size()));
    DFTG_CUDA(cudaMalloc(&c->d_Kt, sizeof(double) * T->Kt.size()));
    DFTG_CUDA(cudaMalloc(&c->d_maps32, sizeof(float) * T->m32.size()));
    DFTG_TRY_L(up(c->d_Gt, T->Gt.data(), sizeof(double) * T->Gt.size()));
    DFTG_TRY_L(up(c->d_Gb, T->Gb.data(), sizeof(double) * T->Gb.size()));
    DFTG_TRY_L(up(c->d_Kt, T->Kt.data(), sizeof(double) * T->Kt.size()));
    DFTG_TRY_L(up(c->d_Y, T->Y.data(), sizeof(double) * T->Y.size()));
    DFTG_TRY_L(up(c->d_Yw, T->Yw.data(), sizeof(double) * T->Yw.size()));
    DFTG_TRY_L(up(c->d_Y32, T->Y32.data(), sizeof(float) * T->Y32.size()));
    DFTG_TRY_L(up(c->d_Ywt32, T->Ywt32.data(), sizeof(float) * T->Ywt32.size()));
    DFTG_TRY_L(up(c->d_pre, T->pre.data(), sizeof(double) * T->pre.size()));
    DFTG_TRY_L(up(c->d_fold, T->fold.data(), sizeof(double) * T->fold.size()));
    DFTG_TRY_L(up(c->d_rec, T->rec.data(), sizeof(double) * T->rec.size()));
    DFTG_TRY_L(up(c->d_pre32, T->pre32.data(), sizeof(float) * T->pre32.size()));
    DFTG_TRY_L(up(c->d_rec32, T->rec32.data(), sizeof(float) * T->rec32.size()));
    DFTG_TRY_L(up(c->d_sx, T->sx.data(), sizeof(double) * N));
    DFTG_TRY_L(up(c->d_splf, T->f.data(), sizeof(double) * T->f.size()));
    DFTG_TRY_L(up(c->d_maps32, T->m32.data(), sizeof(float) * T->m32.size()));
    c->nlebpair = (int)T->pairs.size() / 2;
    if (c->nlebpair > 0) {
        DFTG_CUDA(cudaMalloc(&c->d_lebpair, sizeof(int2) * c->nlebpair));
        DFTG_TRY_L(up(c->d_lebpair, T->pairs.data(), sizeof(int) * T->pairs.size()));
    }
    return DFTG_OK;
}

// ------------------------------------------------------------------ kernels

// K5a (FP64): CTA per (atom, shell)
__global__ void k_rholm(int nrad, int nang, int nlm, int cell0, const double *__restrict__ rho,
                        const double *__restrict__ wb, const double *__restrict__ Yw, double *__restrict__ rholm)
{
    extern __shared__ double s_rw[];   // [nang]
    const int al = blockIdx.x / nrad, i = blockIdx.x % nrad, a = cell0 + al;
    const size_t base = ((size_t)al * nrad + i) * nang;
    for (int j = threadIdx.x; j < nang; j += blockDim.x) s_rw[j] = rho[base + j] * wb[base + j];
    __syncthreads();
    for (int lm = threadIdx.x; lm < nlm; lm += blockDim.x) {
        const double *y = Yw + (size_t)lm * nang;
        double s = 0.0;
        for (int j = 0; j < nang; ++j) s += s_rw[j] * y[j];
        rholm[((size_t)a * nlm + lm) * nrad + i] = s * 4.0 * kPi;
    }
}

// ------------------------------------------------------------------
// Double-float GEMM for the own-cell potential of the mixed multipole step: C = A B with A (M x K) and
// B (K x N) given as FP32 hi + lo planes (row-major, leading dimensions lda /
// ldb), every product formed exactly (TwoProd) and accumulated with TwoSum, so
// C carries ~2^-44 relative error.  Tile 16 x 32 per block of 128 threads, 2 x 2
// outputs per thread; K split over gridDim.z slices whose partial results the
// epilogue functor receives with their slice index.
constexpr int kDgBM = 16, kDgBN = 32, kDgBK = 16;

template <class Epi>
__global__ void __launch_bounds__(128) k_dfgemm(int M, int N, int K, const float *__restrict__ Ah,
                                                const float *__restrict__ Al, int lda, const float *__restrict__ Bh,
                                                const float *__restrict__ Bl, int ldb, Epi epi)
{
    __shared__ float sa[2][kDgBK][kDgBM + 1], sb[2][kDgBK][kDgBN + 1];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;        // ty 0..7
    const int m0 = blockIdx.y * kDgBM, n0 = blockIdx.x * kDgBN;
    const int kchunk = (K + gridDim.z - 1) / gridDim.z;
    const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
    float s[2][2] = {{0.f, 0.f}, {0.f, 0.f}}, e[2][2] = {{0.f, 0.f}, {0.f, 0.f}};
    for (int k0 = kbeg; k0 < kend; k0 += kDgBK) {
        for (int i = threadIdx.x; i < kDgBM * kDgBK; i += 128) {          // A tile, transposed
            const int r = i / kDgBK, kk = i % kDgBK, m = m0 + r, k = k0 + kk;
            const bool ok = m < M && k < kend;
            sa[0][kk][r] = ok ? Ah[(size_t)m * lda + k] : 0.f;
            sa[1][kk][r] = ok ? Al[(size_t)m * lda + k] : 0.f;
        }
        for (int i = threadIdx.x; i < kDgBK * kDgBN; i += 128) {          // B tile
            const int kk = i / kDgBN, c = i % kDgBN, n = n0 + c, k = k0 + kk;
            const bool ok = n < N && k < kend;
            sb[0][kk][c] = ok ? Bh[(size_t)k * ldb + n] : 0.f;
            sb[1][kk][c] = ok ? Bl[(size_t)k * ldb + n] : 0.f;
        }
        __syncthreads();
#pragma unroll 4
        for (int kk = 0; kk < kDgBK; ++kk) {
            const float a0h = sa[0][kk][ty], a0l = sa[1][kk][ty], a1h = sa[0][kk][ty + 8], a1l = sa[1][kk][ty + 8];
            const float b0h = sb[0][kk][tx], b0l = sb[1][kk][tx], b1h = sb[0][kk][tx + 16], b1l = sb[1][kk][tx + 16];
            df_mac(s[0][0], e[0][0], a0h, a0l, b0h, b0l);
            df_mac(s[0][1], e[0][1], a0h, a0l, b1h, b1l);
            df_mac(s[1][0], e[1][0], a1h, a1l, b0h, b0l);
            df_mac(s[1][1], e[1][1], a1h, a1l, b1h, b1l);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int m = m0 + ty + 8 * i, n = n0 + tx + 16 * j;
            if (m < M && n < N) epi(m, n, (int)blockIdx.z, df_norm(s[i][j], e[i][j]));
        }
}

// V_own[p] = (1 / r_p) sum_lm U[a][lm][i] Y_lm[j], p = (a N + i) nang + j
struct EpiVown {
    int nang;
    const double *invr;
    double *Vown;
    __device__ void operator()(int m, int n, int, dfl v) const
    {
        const size_t p = (size_t)m * nang + n;
        Vown[p] = df_to(v) * invr[p];
    }
};

// K5b: U_lm = G_l rho_lm (+ the l = 0 boundary column times q_a): one block per
// (atom, lm), one thread per radial point, four partial sums per dot product.
// Writes U (FP64) and its hi/lo FP32 split.
__global__ void k_poisson(int natoms, int cell0, int nrad, int lmax, const double *__restrict__ Gt,
                          const double *__restrict__ Gb, const double *__restrict__ rholm,
                          const double *__restrict__ scal, double *__restrict__ U, float *__restrict__ U32)
{
    extern __shared__ double s_r[];     // [nrad]
    const int nlm = (lmax + 1) * (lmax + 1);
    const int id = blockIdx.x + cell0 * nlm, a = id / nlm, lm = id % nlm, N = nrad;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) ++l;
    const double *R = rholm + (size_t)id * N;
    for (int k = threadIdx.x; k < N; k += blockDim.x) s_r[k] = R[k];
    __syncthreads();
    const double *G = Gt + (size_t)l * N * N;
    const double q = (lm == 0) ? scal[kScalAtomQ + a] : 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        int k = 0;
        for (; k + 3 < N; k += 4) {
            s0 += G[(size_t)k * N + i] * s_r[k];
            s1 += G[(size_t)(k + 1) * N + i] * s_r[k + 1];
            s2 += G[(size_t)(k + 2) * N + i] * s_r[k + 2];
            s3 += G[(size_t)(k + 3) * N + i] * s_r[k + 3];
        }
        for (; k < N; ++k) s0 += G[(size_t)k * N + i] * s_r[k];
        double v = (s0 + s1) + (s2 + s3);
        if (lm == 0) v += Gb[i] * q;
        U[(size_t)id * N + i] = v;
        const float hi = (float)v;
        U32[(size_t)id * N + i] = hi;
        U32[(size_t)natoms * nlm * N + (size_t)id * N + i] = (float)(v - (double)hi);
    }
}

// K5c (FP64): own-cell potential for every point
__global__ void k_vown(size_t npts, int nrad, int nang, int nlm, int cell0, const double *__restrict__ rn,
                       const double *__restrict__ leb, const double *__restrict__ Y, const double *__restrict__ U,
                       double *__restrict__ Vown)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int per_atom = nrad * nang;
    const int a = cell0 + (int)(p / per_atom), rem = (int)(p % per_atom), i = rem / nang, j = rem % nang;
    const double ri = rn[i];
    const double px = leb[4 * j] * ri, py = leb[4 * j + 1] * ri, pz = leb[4 * j + 2] * ri;
    const double inv_r = 1.0 / sqrt(px * px + py * py + pz * pz);
    const double *u = U + (size_t)a * nlm * nrad + i;
    double v = 0.0;
    for (int lm = 0; lm < nlm; ++lm) v += inv_r * Y[(size_t)lm * nang + j] * u[(size_t)lm * nrad];
    Vown[p] = v;
}


// K5d: spline coefficients of U_lm over increasing r (cspline.cpp:66-142):
// derivatives D = K y with the precomputed x-only map K, then the per-interval
// cubic coefficients.  One block per (atom, lm).  Writes the FP64 table
// [atom][lm][interval][4] and the mixed table [atom][lm][interval][8] =
// fold_lm * (c0..c3) split into FP32 hi and lo.
__global__ void k_splines(int natoms, int cell0, int nrad, int nlm, const double *__restrict__ splf,
                          const double *__restrict__ Kt, const double *__restrict__ U,
                          const double *__restrict__ fold, double *__restrict__ spl, float *__restrict__ splm)
{
    extern __shared__ double s_spl[];   // y [n], D [n]
    const int id = blockIdx.x + cell0 * nlm, n = nrad;
    double *y = s_spl, *D = s_spl + n;
    const double *u = U + (size_t)id * n;      // u[i] at r_n[i] (decreasing r)
    for (int i = threadIdx.x; i < n; i += blockDim.x) y[i] = u[n - 1 - i];
    __syncthreads();
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double s0 = 0.0, s1 = 0.0;
        int j = 0;
        for (; j + 1 < n; j += 2) {
            s0 += Kt[(size_t)j * n + i] * y[j];
            s1 += Kt[(size_t)(j + 1) * n + i] * y[j + 1];
        }
        if (j < n) s0 += Kt[(size_t)j * n + i] * y[j];
        D[i] = s0 + s1;
    }
    __syncthreads();
    const double *inv_h = splf;
    const int lm = id % nlm;
    const double F = fold[lm];
    double *out = spl + (size_t)id * n * 4;
    float *o32 = splm + (size_t)id * n * 8;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        double cc[4];
        if (i < n - 1) {
            const double dx = inv_h[i];
            const double dy = (y[i + 1] - y[i]) * dx;
            cc[0] = y[i];
            cc[1] = D[i];
            cc[2] = dx * (3 * dy - 2 * D[i] - D[i + 1]);
            cc[3] = dx * dx * (-2 * dy + D[i] + D[i + 1]);
        } else {                     // clamp value of the last knot
            cc[0] = y[n - 1]; cc[1] = 0.0; cc[2] = 0.0; cc[3] = 0.0;
        }
        for (int k = 0; k < 4; ++k) {
            out[4 * i + k] = cc[k];
            const double v = F * cc[k];
            const float hi = (float)v;
            o32[8 * i + k] = hi;
            o32[8 * i + 4 + k] = (float)(v - (double)hi);
        }
    }
}

// K5a-d (mixed, one launch): the multipole chain of one atom cell for a group
// of kMpLG (l, m) rows per CTA: rho_lm (atomicgrid.cpp:241-296), the radial
// Poisson map with the l = 0 boundary value sqrt(4 pi) q_a (atomicgrid.cpp:
// 301-432), and the spline fit of U_lm (atomicgrid.cpp:535-556), all in
// double-float arithmetic with exact products.  The CTA stages the cell's
// rho w_becke (the FP32 hi / lo planes of the point kernel when given, else
// formed from the FP64 arrays) kMpSC shells per pass, and each thread forms
// one rho_lm(i) as a dot product over the Lebedev points against the group's
// w_leb Y_lm rows, so nothing is reduced across threads.  The Poisson map of
// each l and the spline derivative map are then staged in the same shared
// memory (when an N x N double-float map fits) and applied a row per thread.
// The CTA holding lm = 0 also sums q_a = sum w rho over the cell (FP64, fixed
// order) for the boundary value.  Writes U (FP64 and split FP32, both radial
// orders) and the spline tables.
constexpr int kMpLG = 4;          // (l, m) rows per CTA
constexpr int kMpSC = 32;         // radial shells staged per pass
constexpr int kMpThreads = 320;

static size_t mp_stage_bytes(int nang) { return sizeof(dfl) * (size_t)kMpSC * (size_t)(nang | 1); }

size_t multipole_smem(int nrad, int nang)
{
    return mp_stage_bytes(nang) + sizeof(dfl) * ((size_t)kMpLG * nang + 3 * (size_t)kMpLG * nrad) +
           64 * sizeof(double);
}

// acc = sum_k M[k][i] x[k] over k < N (M given as hi / lo planes with row
// stride N): four independent compensated accumulators (exact leading
// products by TwoProd, the cross terms and the roundings gathered in the error
// part), normalised once at the end
__device__ __forceinline__ dfl mp_matvec(const float *__restrict__ Mh, const float *__restrict__ Ml, int N, int i,
                                         const dfl *__restrict__ x, bool reverse_x)
{
    float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f, s2 = 0.f, e2 = 0.f, s3 = 0.f, e3 = 0.f;
    int k = 0;
    for (; k + 3 < N; k += 4) {
        const dfl x0 = reverse_x ? x[N - 1 - k] : x[k], x1 = reverse_x ? x[N - 2 - k] : x[k + 1];
        const dfl x2 = reverse_x ? x[N - 3 - k] : x[k + 2], x3 = reverse_x ? x[N - 4 - k] : x[k + 3];
        df_mac(s0, e0, Mh[(size_t)k * N + i], Ml[(size_t)k * N + i], x0.h, x0.l);
        df_mac(s1, e1, Mh[(size_t)(k + 1) * N + i], Ml[(size_t)(k + 1) * N + i], x1.h, x1.l);
        df_mac(s2, e2, Mh[(size_t)(k + 2) * N + i], Ml[(size_t)(k + 2) * N + i], x2.h, x2.l);
        df_mac(s3, e3, Mh[(size_t)(k + 3) * N + i], Ml[(size_t)(k + 3) * N + i], x3.h, x3.l);
    }
    for (; k < N; ++k) {
        const dfl xk = reverse_x ? x[N - 1 - k] : x[k];
        df_mac(s0, e0, Mh[(size_t)k * N + i], Ml[(size_t)k * N + i], xk.h, xk.l);
    }
    return df_add(df_add(df_norm(s0, e0), df_norm(s1, e1)), df_add(df_norm(s2, e2), df_norm(s3, e3)));
}

// n floats global -> shared as asynchronous 4-byte copies, all in flight at
// once (no register staging); complete after mp_copy_wait
__device__ __forceinline__ void mp_copy(float *__restrict__ dst, const float *__restrict__ src, int n)
{
    for (int e = threadIdx.x; e < n; e += kMpThreads)
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"((uint32_t)__cvta_generic_to_shared(dst + e)),
                     "l"(src + e)
                     : "memory");
}
// this thread's copies landed (then a __syncthreads for the others')
__device__ __forceinline__ void mp_copy_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

__device__ __forceinline__ void multipole_block(const MpArgs A, int vb)
{
    const int natoms = A.natoms, cell0 = A.cell0, N = A.N, nang = A.nang, lmax = A.lmax, ngroup = A.ngroup;
    const float *__restrict__ rw32 = A.rw32;
    const size_t npad = A.npad;
    const double *__restrict__ rho = A.rho, *__restrict__ wb = A.wb, *__restrict__ w = A.w;
    const float *__restrict__ Ywt32 = A.Ywt32, *__restrict__ maps = A.maps;
    double *__restrict__ scal = A.scal, *__restrict__ U = A.U;
    float *__restrict__ U32 = A.U32, *__restrict__ U32T = A.U32T;
    const int want64 = A.want64;
    double *__restrict__ spl = A.spl;
    float *__restrict__ splm = A.splm;
    extern __shared__ __align__(16) unsigned char mp_smem[];
    const int nlm = (lmax + 1) * (lmax + 1);
    const int row = nang | 1;
    const size_t stage_bytes = sizeof(dfl) * (size_t)kMpSC * row;
    dfl *sRW = reinterpret_cast<dfl *>(mp_smem);                 // [kMpSC][row] rho w_becke
    float *sMap = reinterpret_cast<float *>(mp_smem);            // the same space: a map's hi, lo planes
    const bool stage_maps = (size_t)2 * N * N * sizeof(float) <= stage_bytes;
    dfl *sY = reinterpret_cast<dfl *>(mp_smem + stage_bytes);    // [kMpLG][nang] w_leb Y_lm
    dfl *sR = sY + (size_t)kMpLG * nang;                         // [kMpLG][N] rho_lm
    dfl *sU = sR + (size_t)kMpLG * N;                            // [kMpLG][N] U_lm
    dfl *sD = sU + (size_t)kMpLG * N;                            // [kMpLG][N] spline derivatives
    double *sred = reinterpret_cast<double *>(sD + (size_t)kMpLG * N);
    const int tid = threadIdx.x;
    const int al = vb / ngroup, g = vb % ngroup, a = cell0 + al;
    // group g: rows lm0 .. lm0 + nl - 1 of one degree l (at most kMpLG of them)
    int lm0 = 0, nl = 0;
    for (int l = 0, gg = g; l <= lmax; ++l) {
        const int nrow = 2 * l + 1, ngl = (nrow + kMpLG - 1) / kMpLG;
        if (gg < ngl) {
            lm0 = l * l + gg * kMpLG;
            nl = min(kMpLG, nrow - gg * kMpLG);
            break;
        }
        gg -= ngl;
    }
    const size_t base = (size_t)al * N * nang;
    const size_t uhalf = (size_t)natoms * nlm * N;
    // w_leb Y_lm at the first direction of every antipodal pair: [row][pair]
    const int npair = A.npair;
    const int2 *__restrict__ pairs = A.pairs;
    for (int e = tid; e < nl * npair; e += kMpThreads) {
        const int r = e / npair, j = __ldg(&pairs[e % npair].x);
        sY[e] = dfl{Ywt32[(size_t)j * nlm + lm0 + r], Ywt32[(size_t)nang * nlm + (size_t)j * nlm + lm0 + r]};
    }
    // q_a for the boundary row of lm = 0 (four loads in flight per thread)
    double q = 0.0;
    if (lm0 == 0) {
        const int n = N * nang;
        double t0 = 0.0, t1 = 0.0, t2 = 0.0, t3 = 0.0;
        int e = tid;
        for (; e + 3 * kMpThreads < n; e += 4 * kMpThreads) {
            t0 += w[base + e] * rho[base + e];
            t1 += w[base + e + kMpThreads] * rho[base + e + kMpThreads];
            t2 += w[base + e + 2 * kMpThreads] * rho[base + e + 2 * kMpThreads];
            t3 += w[base + e + 3 * kMpThreads] * rho[base + e + 3 * kMpThreads];
        }
        for (; e < n; e += kMpThreads) t0 += w[base + e] * rho[base + e];
        q = block_sum((t0 + t1) + (t2 + t3), sred);
        if (tid == 0) {
            sred[32] = q;
            scal[kScalAtomQ + a] = q;
        }
    }
    const dfl four_pi = df_from(4.0 * kPi);
    for (int i0 = 0; i0 < N; i0 += kMpSC) {
        const int ns = min(kMpSC, N - i0);
        __syncthreads();                                          // the previous pass is done with sRW
        // a thread per (antipodal pair (j, a), eight shells), the shells' loads in
        // flight: the even and odd combinations rho w(j) +- rho w(a)
        // (Y_lm(a) = (-1)^l Y_lm(j))
        const int nb8 = (ns + 7) / 8;
        for (int item = tid; item < npair * nb8; item += kMpThreads) {
            const int k = item % npair, ii0 = (item / npair) * 8;
            const int2 ja = __ldg(&pairs[k]);
            {
                dfl v[8], w[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const size_t p = base + (size_t)(i0 + min(ii0 + u, ns - 1)) * nang;
                    const size_t pj = p + ja.x, pa = p + ja.y;
                    v[u] = rw32 ? dfl{rw32[pj], rw32[npad + pj]} : df_from(rho[pj] * wb[pj]);
                    w[u] = rw32 ? dfl{rw32[pa], rw32[npad + pa]} : df_from(rho[pa] * wb[pa]);
                }
#pragma unroll
                for (int u = 0; u < 8; ++u)
                    if (ii0 + u < ns) {
                        sRW[(size_t)(ii0 + u) * row + k] = df_add(v[u], w[u]);
                        sRW[(size_t)(ii0 + u) * row + npair + k] = df_sub(v[u], w[u]);
                    }
            }
        }
        __syncthreads();
        // two threads per rho_lm(i), each over half of the pairs, met by a
        // shuffle; every lane of a warp takes part (items past the end run on
        // empty ranges).  Row lm of degree l takes the even combinations for
        // even l, the odd ones for odd l.
        const int nitem = 2 * nl * ns;
        const int half_pair = (npair + 1) / 2;
        for (int o0 = (tid & ~31); o0 < nitem; o0 += kMpThreads) {
            const int o = o0 + (tid & 31);
            const bool valid = o < nitem;
            const int out = o >> 1, hf = o & 1;
            const int r = valid ? out % nl : 0, ii = valid ? out / nl : 0;
            const int j0 = hf ? half_pair : 0, j1 = valid ? (hf ? npair : half_pair) : 0;
            int l = 0;
            while ((l + 1) * (l + 1) <= lm0 + r) ++l;
            const dfl *x = sRW + (size_t)ii * row + ((l & 1) ? npair : 0), *y = sY + (size_t)r * npair;
            float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f, s2 = 0.f, e2 = 0.f, s3 = 0.f, e3 = 0.f;
            int j = j0;
            for (; j + 3 < j1; j += 4) {
                df_mac(s0, e0, x[j].h, x[j].l, y[j].h, y[j].l);
                df_mac(s1, e1, x[j + 1].h, x[j + 1].l, y[j + 1].h, y[j + 1].l);
                df_mac(s2, e2, x[j + 2].h, x[j + 2].l, y[j + 2].h, y[j + 2].l);
                df_mac(s3, e3, x[j + 3].h, x[j + 3].l, y[j + 3].h, y[j + 3].l);
            }
            for (; j < j1; ++j) df_mac(s0, e0, x[j].h, x[j].l, y[j].h, y[j].l);
            dfl t = df_add(df_add(df_norm(s0, e0), df_norm(s1, e1)), df_add(df_norm(s2, e2), df_norm(s3, e3)));
            const dfl u{__shfl_xor_sync(0xffffffffu, t.h, 1), __shfl_xor_sync(0xffffffffu, t.l, 1)};
            t = hf ? df_add(u, t) : df_add(t, u);         // the same order in both lanes
            if (valid && hf == 0) sR[r * N + i0 + ii] = df_mul(t, four_pi);
        }
    }
    __syncthreads();
    if (lm0 == 0) q = sred[32];
    // Poisson: U = G_l rho_lm (+ Gb q for lm = 0), one l of the group at a time
    const size_t ng = (size_t)(lmax + 1) * N * N;
    const float *Gbh = maps + 2 * ng, *Gbl = Gbh + N;
    int lfirst = 0, llast = 0;
    while ((lfirst + 1) * (lfirst + 1) <= lm0) ++lfirst;
    while ((llast + 1) * (llast + 1) <= lm0 + nl - 1) ++llast;
    for (int l = lfirst; l <= llast; ++l) {
        const float *Gh = maps + (size_t)l * N * N, *Gl = Gh + ng;
        if (stage_maps) {
            __syncthreads();                                      // sMap free (rho w planes or the previous l)
            mp_copy(sMap, Gh, N * N);
            mp_copy(sMap + (size_t)N * N, Gl, N * N);
            mp_copy_wait();
            __syncthreads();
            Gh = sMap;
            Gl = sMap + (size_t)N * N;
        }
        for (int o = tid; o < nl * N; o += kMpThreads) {
            const int r = o / N, i = o % N, lm = lm0 + r;
            if (lm < l * l || lm > l * l + 2 * l) continue;
            dfl v = mp_matvec(Gh, Gl, N, i, sR + r * N, false);
            if (lm == 0) v = df_fma(v, dfl{Gbh[i], Gbl[i]}, df_from(q));
            sU[r * N + i] = v;
            const size_t id = (size_t)a * nlm + lm;
            U[id * N + i] = df_to(v);
            U32[id * N + i] = v.h;
            U32[uhalf + id * N + i] = v.l;
            U32T[((size_t)a * N + i) * nlm + lm] = v.h;
            U32T[uhalf + ((size_t)a * N + i) * nlm + lm] = v.l;
        }
    }
    // spline derivatives over increasing r: D = K y, y[i] = U[N - 1 - i]
    const float *Kh = maps + 2 * ng + 2 * (size_t)N, *Kl = Kh + (size_t)N * N;
    const float *ih = Kl + (size_t)N * N, *il = ih + N;
    const float *fh = il + N, *fl = fh + nlm;
    __syncthreads();                                              // sU complete; sMap free
    if (stage_maps) {
        mp_copy(sMap, Kh, N * N);
        mp_copy(sMap + (size_t)N * N, Kl, N * N);
        mp_copy_wait();
        __syncthreads();
        Kh = sMap;
        Kl = sMap + (size_t)N * N;
    }
    for (int o = tid; o < nl * N; o += kMpThreads) {
        const int r = o / N, i = o % N;
        sD[r * N + i] = mp_matvec(Kh, Kl, N, i, sU + r * N, true);
    }
    __syncthreads();
    for (int o = tid; o < nl * N; o += kMpThreads) {
        const int r = o / N, i = o % N, lm = lm0 + r;
        const dfl *u = sU + r * N, *D = sD + r * N;
        const dfl F{fh[lm], fl[lm]};
        dfl cc[4];
        if (i < N - 1) {
            const dfl dx{ih[i], il[i]}, y0 = u[N - 1 - i], y1 = u[N - 2 - i];
            const dfl D0 = D[i], D1 = D[i + 1];
            const dfl dy = df_mul(df_sub(y1, y0), dx);
            const dfl three{3.f, 0.f}, two{2.f, 0.f};
            cc[0] = y0;
            cc[1] = D0;
            cc[2] = df_mul(dx, df_sub(df_sub(df_mul(three, dy), df_mul(two, D0)), D1));
            cc[3] = df_mul(df_mul(dx, dx), df_add(df_add(df_mul(dfl{-2.f, 0.f}, dy), D0), D1));
        } else {                     // clamp value of the last knot
            cc[0] = u[0];
            cc[1] = cc[2] = cc[3] = dfl{0.f, 0.f};
        }
        const size_t id = (size_t)a * nlm + lm;
        float *o32 = splm + (id * N + i) * 8;
        for (int k = 0; k < 4; ++k) {
            const dfl v = df_mul(F, cc[k]);
            o32[k] = v.h;
            o32[4 + k] = v.l;
            if (want64) spl[(id * N + i) * 4 + k] = df_to(cc[k]);
        }
    }
}

__global__ void __launch_bounds__(kMpThreads, 2) k_multipole(const MpArgs a)
{
    pdl_wait();
    multipole_block(a, (int)blockIdx.x);
    pdl_signal();
}

__global__ void __launch_bounds__(kMpThreads, 2) k_multipole_group(const MpArgs *__restrict__ args, GroupQueue q)
{
    __shared__ int s_item;
    gq_run(q, &s_item, [&](int m, int vb, int) {
        const MpArgs a = args[m];
        multipole_block(a, vb);
        return true;
    });
}

// spline interval of r: smallest i >= 1 with r <= sx[i] (cspline.cpp:163-170),
// from the analytic inverse of the radial map and an exact comparison fix-up
__device__ __forceinline__ void spline_interval(double rd, const double *__restrict__ sx, int N, double fscale,
                                                int &iv, double &t)
{
    if (rd < sx[0]) { iv = 0; t = 0.0; return; }
    if (rd >= sx[N - 1]) { iv = N - 1; t = 0.0; return; }
    const float pr = acosf((float)((rd - 1.0) / (rd + 1.0))) * (float)fscale;
    int i = (int)ceilf((float)N - pr);
    i = max(1, min(N - 1, i));
    while (i < N - 1 && rd > sx[i]) ++i;
    while (i > 1 && rd <= sx[i - 1]) --i;
    iv = i - 1;
    t = rd - sx[iv];
}

// K5e (FP64): total potential on every point; writes V and cj = w V / 2
__global__ void __launch_bounds__(128) k_vcross64(size_t npts, size_t npad, int natoms, int cell0, int nrad, int nang,
                                                  int lmax,
                                                  const double *__restrict__ atoms, const double *__restrict__ X,
                                                  const double *__restrict__ Yc, const double *__restrict__ Zc,
                                                  const double *__restrict__ W, const double *__restrict__ sx,
                                                  const double *__restrict__ spl, const double *__restrict__ pre,
                                                  const double *__restrict__ rec, const double *__restrict__ Vown,
                                                  double *__restrict__ V, double *__restrict__ cj,
                                                  float *__restrict__ cj32)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    if (p >= npts) { V[p] = 0.0; cj[p] = 0.0; cj32[p] = 0.f; return; }
    const int nlm = (lmax + 1) * (lmax + 1);
    const int N = nrad;
    const int a = cell0 + (int)(p / ((size_t)nrad * nang));
    const double px = X[p], py = Yc[p], pz = Zc[p];
    const double fscale = (double)(N + 1) / kPi;
    double Vt = 0.0;
    for (int k = 0; k < natoms; ++k) {
        if (k == a) { Vt += Vown[p]; continue; }
        const double dx = px - atoms[4 * k], dy = py - atoms[4 * k + 1], dz = pz - atoms[4 * k + 2];
        const double r = sqrt(dx * dx + dy * dy + dz * dz);
        int iv;
        double t;
        spline_interval(r, sx, N, fscale, iv, t);
        const double inv_r = 1.0 / r;
        const double ux = dx * inv_r, uy = dy * inv_r, uz = dz * inv_r;
        const double *cf = spl + ((size_t)k * nlm * N + iv) * 4;
        double acc = 0.0, cm = 1.0, sm = 0.0, qmm = 1.0;
        for (int m = 0; m <= lmax; ++m) {
            double q2 = 0.0, q1 = qmm;
            for (int l = m; l <= lmax; ++l) {
                double q;
                if (l == m) q = qmm;
                else {
                    const int lmi = l * l + l + m;
                    q = rec[2 * lmi] * uz * q1 - rec[2 * lmi + 1] * q2;
                    q2 = q1;
                    q1 = q;
                }
                const int lp = l * l + l + m;
                const double *c0 = cf + (size_t)lp * N * 4;
                const double sp = c0[0] + t * (c0[1] + t * (c0[2] + t * c0[3]));
                if (m == 0) {
                    acc += pre[lp] * q * sp;
                } else {
                    const int ln = l * l + l - m;
                    const double *c1 = cf + (size_t)ln * N * 4;
                    const double sn = c1[0] + t * (c1[1] + t * (c1[2] + t * c1[3]));
                    acc += pre[lp] * q * cm * sp + pre[ln] * q * sm * sn;
                }
            }
            const double cn = cm * ux - sm * uy, sn2 = cm * uy + sm * ux;
            cm = cn;
            sm = sn2;
            qmm = -(double)(2 * m + 1) * qmm;
        }
        Vt += inv_r * acc;
    }
    V[p] = Vt;
    const double c = 0.5 * (W[p] * Vt);
    cj[p] = c;
    cj32[p] = (float)c;
}

// S_lm = prod_{j = |m| + 1}^{l} (2 j - 1) at lm = l^2 + l + m, l <= kLmaxCap: the
// scale between the integer recursion R_l^|m| and its monic form (exact in FP32
// up to l = 8, rounded once above)
__constant__ float kLegScale[(kLmaxCap + 1) * (kLmaxCap + 1)] = {
    1.f, 1.f, 1.f, 1.f, 1.f, 3.f,
    3.f, 3.f, 1.f, 1.f, 5.f, 15.f,
    15.f, 15.f, 5.f, 1.f, 1.f, 7.f,
    35.f, 105.f, 105.f, 105.f, 35.f, 7.f,
    1.f, 1.f, 9.f, 63.f, 315.f, 945.f,
    945.f, 945.f, 315.f, 63.f, 9.f, 1.f,
    1.f, 11.f, 99.f, 693.f, 3465.f, 10395.f,
    10395.f, 10395.f, 3465.f, 693.f, 99.f, 11.f,
    1.f, 1.f, 13.f, 143.f, 1287.f, 9009.f,
    45045.f, 135135.f, 135135.f, 135135.f, 45045.f, 9009.f,
    1287.f, 143.f, 13.f, 1.f, 1.f, 15.f,
    195.f, 2145.f, 19305.f, 135135.f, 675675.f, 2027025.f,
    2027025.f, 2027025.f, 675675.f, 135135.f, 19305.f, 2145.f,
    195.f, 15.f, 1.f, 1.f, 17.f, 255.f,
    3315.f, 36465.f, 328185.f, 2297295.f, 11486475.f, 3.445942500e+07f,
    3.445942500e+07f, 3.445942500e+07f, 11486475.f, 2297295.f, 328185.f, 36465.f,
    3315.f, 255.f, 17.f, 1.f, 1.f, 19.f,
    323.f, 4845.f, 62985.f, 692835.f, 6235515.f, 4.364860500e+07f,
    2.182430250e+08f, 6.547290750e+08f, 6.547290750e+08f, 6.547290750e+08f, 2.182430250e+08f, 4.364860500e+07f,
    6235515.f, 692835.f, 62985.f, 4845.f, 323.f, 19.f,
    1.f, 1.f, 21.f, 399.f, 6783.f, 101745.f,
    1322685.f, 14549535.f, 1.309458150e+08f, 9.166207050e+08f, 4.583103525e+09f, 1.374931058e+10f,
    1.374931058e+10f, 1.374931058e+10f, 4.583103525e+09f, 9.166207050e+08f, 1.309458150e+08f, 14549535.f,
    1322685.f, 101745.f, 6783.f, 399.f, 21.f, 1.f,
    1.f, 23.f, 483.f, 9177.f, 156009.f, 2340135.f,
    3.042175500e+07f, 3.346393050e+08f, 3.011753745e+09f, 2.108227622e+10f, 1.054113811e+11f, 3.162341432e+11f,
    3.162341432e+11f, 3.162341432e+11f, 1.054113811e+11f, 2.108227622e+10f, 3.011753745e+09f, 3.346393050e+08f,
    3.042175500e+07f, 2340135.f, 156009.f, 9177.f, 483.f, 23.f,
    1.f, 1.f, 25.f, 575.f, 12075.f, 229425.f,
    3900225.f, 5.850337500e+07f, 7.605438750e+08f, 8.365982625e+09f, 7.529384362e+10f, 5.270569054e+11f,
    2.635284527e+12f, 7.905853581e+12f, 7.905853581e+12f, 7.905853581e+12f, 2.635284527e+12f, 5.270569054e+11f,
    7.529384362e+10f, 8.365982625e+09f, 7.605438750e+08f, 5.850337500e+07f, 3900225.f, 229425.f,
    12075.f, 575.f, 25.f, 1.f, 1.f, 27.f,
    675.f, 15525.f, 326025.f, 6194475.f, 1.053060750e+08f, 1.579591125e+09f,
    2.053468462e+10f, 2.258815309e+11f, 2.032933778e+12f, 1.423053645e+13f, 7.115268223e+13f, 2.134580467e+14f,
    2.134580467e+14f, 2.134580467e+14f, 7.115268223e+13f, 1.423053645e+13f, 2.032933778e+12f, 2.258815309e+11f,
    2.053468462e+10f, 1.579591125e+09f, 1.053060750e+08f, 6194475.f, 326025.f, 15525.f,
    675.f, 27.f, 1.f, 1.f, 29.f, 783.f,
    19575.f, 450225.f, 9454725.f, 1.796397750e+08f, 3.053876175e+09f, 4.580814262e+10f,
    5.955058541e+11f, 6.550564395e+12f, 5.895507956e+13f, 4.126855569e+14f, 2.063427785e+15f, 6.190283354e+15f,
    6.190283354e+15f, 6.190283354e+15f, 2.063427785e+15f, 4.126855569e+14f, 5.895507956e+13f, 6.550564395e+12f,
    5.955058541e+11f, 4.580814262e+10f, 3.053876175e+09f, 1.796397750e+08f, 9454725.f, 450225.f,
    19575.f, 783.f, 29.f, 1.f, 1.f, 31.f,
    899.f, 24273.f, 606825.f, 13956975.f, 2.930964750e+08f, 5.568833025e+09f,
    9.467016142e+10f, 1.420052421e+12f, 1.846068148e+13f, 2.030674963e+14f, 1.827607466e+15f, 1.279325226e+16f,
    6.396626132e+16f, 1.918987840e+17f, 1.918987840e+17f, 1.918987840e+17f, 6.396626132e+16f, 1.279325226e+16f,
    1.827607466e+15f, 2.030674963e+14f, 1.846068148e+13f, 1.420052421e+12f, 9.467016142e+10f, 5.568833025e+09f,
    2.930964750e+08f, 13956975.f, 606825.f, 24273.f, 899.f, 31.f,
    1.f,
};

constexpr int kCrossPerThread = 2;               // pairs per thread of k_vcross_bins
constexpr int kCrossTask = 128 * kCrossPerThread;  // pairs per block
// low halves of the spline coefficients are evaluated for l <= kCrossLoLmax:
// beyond l = 0 they change E_tot of benzene / 6-31G by < 1e-9 Ha
constexpr int kCrossLoLmax = 0;

// K5e (mixed): FP32 recursion with exact integer coefficients; the spline
// coefficients (which carry the Y_lm normalisation) enter as split FP32 hi/lo
// pairs so no rounding is common to all points.  No FP64 work in the pair
// loop: the per-atom contributions accumulate in an FP32 TwoSum pair and meet
// the FP64 own-cell part once per point.
// One block per task: up to 128 P consecutive (point, other atom) pairs of one
// bin (atom k, spline interval iv).  The pairs are ordered by bin once per
// grid, so the bin's spline coefficients are staged once in shared memory and
// each thread evaluates P pairs against them (every coefficient read serves P
// pairs).  The high halves of the coefficients are used for every l, the low
// halves for l <= kCrossLoLmax.  Writes each pair's contribution as an FP32 (hi, lo)
// pair.
template <int P, int LMAX>
__device__ __forceinline__ void vcross_bins_block(const VcbArgs A, int vb)
{
    const int nrad = A.nrad, lmax_rt = A.lmax;
    const int4 *__restrict__ tasks = A.tasks;
    const float4 *__restrict__ pgeo = A.pgeo;
    const float2 *__restrict__ ptk = A.ptk;
    const float *__restrict__ splm = A.splm;
    float2 *__restrict__ out = A.out;
    extern __shared__ float4 s_cf[];      // [nlm][2]: (c0..c3) high, (c0..c3) low
    const int4 task = tasks[vb];  // start, count, atom k, interval iv
    const int lmax = LMAX >= 0 ? LMAX : lmax_rt;   // compile-time for the common cut-offs
    const int nlm = (lmax + 1) * (lmax + 1);
    float ux[P], uy[P], uz[P], ir[P], t[P];
#pragma unroll
    for (int j = 0; j < P; ++j) {
        const int o = threadIdx.x + j * 128;
        if (o < task.y) {
            const float4 g = pgeo[(size_t)task.x + o];
            ux[j] = g.x; uy[j] = g.y; uz[j] = g.z; ir[j] = g.w;
            t[j] = ptk[(size_t)task.x + o].x;
        } else {
            ux[j] = 0.f; uy[j] = 0.f; uz[j] = 1.f; ir[j] = 0.f; t[j] = 0.f;
        }
    }
    // the pair geometry above is fixed per grid; the coefficients come from the
    // multipole kernel
    pdl_wait();
    // the high halves scaled by S_lm = prod_{j = |m| + 1}^{l} (2 j - 1), the
    // scale of the recursion below (one rounding; the low halves are used for
    // l = 0 only, where S = 1)
    for (int i = threadIdx.x; i < 2 * nlm; i += blockDim.x) {
        const int lm = i >> 1;
        float4 c = reinterpret_cast<const float4 *>(splm + (((size_t)task.z * nlm + lm) * nrad + task.w) * 8)[i & 1];
        if ((i & 1) == 0) {
            const float sc = kLegScale[lm];
            c = make_float4(c.x * sc, c.y * sc, c.z * sc, c.w * sc);
        }
        s_cf[i] = c;
    }
    __syncthreads();
    float ah[P], al[P], cm[P], sm[P];
#pragma unroll
    for (int j = 0; j < P; ++j) { ah[j] = 0.f; al[j] = 0.f; cm[j] = 1.f; sm[j] = 0.f; }
#pragma unroll
    for (int m = 0; m <= lmax; ++m) {
        // for m > 0: sum_l q_l s_lm and sum_l q_l s_l,-m first, then times cos m phi
        // and sin m phi once per m
        float r1[P], r2[P], am[P], bm[P];
#pragma unroll
        for (int j = 0; j < P; ++j) { r1[j] = 1.f; r2[j] = 0.f; am[j] = 0.f; bm[j] = 0.f; }
#pragma unroll
        for (int l = m; l <= lmax; ++l) {
            float q[P];
            // the recursion R_l = (2l-1) z R_{l-1} - (l+m-1)(l-m-1) R_{l-2} divided by
            // S_l = prod (2j-1): Q_l = z Q_{l-1} - beta_l Q_{l-2}, Q_m = 1, Q_{m+1} = z
            if (l == m) {
#pragma unroll
                for (int j = 0; j < P; ++j) q[j] = 1.f;
            } else if (l == m + 1) {
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    q[j] = uz[j];
                    r2[j] = r1[j];
                    r1[j] = q[j];
                }
            } else {
                const float beta = (float)((double)((l + m - 1) * (l - m - 1)) / ((double)(2 * l - 1) * (double)(2 * l - 3)));
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    q[j] = fmaf(uz[j], r1[j], -beta * r2[j]);
                    r2[j] = r1[j];
                    r1[j] = q[j];
                }
            }
            const bool lo = l <= kCrossLoLmax;
            const float4 ch = s_cf[2 * (l * l + l + m)];
            const float4 cl = lo ? s_cf[2 * (l * l + l + m) + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
            if (m == 0) {
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    const float sh = fmaf(t[j], fmaf(t[j], fmaf(t[j], ch.w, ch.z), ch.y), ch.x);
                    ah[j] = fmaf(q[j], sh, ah[j]);
                    if (lo) {
                        const float sl = fmaf(t[j], fmaf(t[j], fmaf(t[j], cl.w, cl.z), cl.y), cl.x);
                        al[j] = fmaf(q[j], sl, al[j]);
                    }
                }
            } else {
                const float4 dh = s_cf[2 * (l * l + l - m)];
                const float4 dl = lo ? s_cf[2 * (l * l + l - m) + 1] : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
                for (int j = 0; j < P; ++j) {
                    const float sh = fmaf(t[j], fmaf(t[j], fmaf(t[j], ch.w, ch.z), ch.y), ch.x);
                    const float nh = fmaf(t[j], fmaf(t[j], fmaf(t[j], dh.w, dh.z), dh.y), dh.x);
                    am[j] = fmaf(q[j], sh, am[j]);
                    bm[j] = fmaf(q[j], nh, bm[j]);
                    if (lo) {
                        const float qc = q[j] * cm[j], qs = q[j] * sm[j];
                        const float sl = fmaf(t[j], fmaf(t[j], fmaf(t[j], cl.w, cl.z), cl.y), cl.x);
                        const float nl = fmaf(t[j], fmaf(t[j], fmaf(t[j], dl.w, dl.z), dl.y), dl.x);
                        al[j] = fmaf(qc, sl, fmaf(qs, nl, al[j]));
                    }
                }
            }
        }
        if (m > 0) {
#pragma unroll
            for (int j = 0; j < P; ++j) ah[j] = fmaf(cm[j], am[j], fmaf(sm[j], bm[j], ah[j]));
        }
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const float cn = cm[j] * ux[j] - sm[j] * uy[j], sn = cm[j] * uy[j] + sm[j] * ux[j];
            cm[j] = cn;
            sm[j] = sn;
        }
    }
#pragma unroll
    for (int j = 0; j < P; ++j) {
        const int o = threadIdx.x + j * 128;
        if (o < task.y) {
            const float vh = ir[j] * ah[j];
            const float vl = fmaf(ir[j], ah[j], -vh) + ir[j] * al[j];
            out[(size_t)task.x + o] = make_float2(vh, vl);
        }
    }
}

template <int P, int LMAX>
__global__ void __launch_bounds__(128) k_vcross_bins(const VcbArgs a)
{
    vcross_bins_block<P, LMAX>(a, (int)blockIdx.x);
    pdl_signal();
}

template <int P, int LMAX>
__global__ void __launch_bounds__(128) k_vcross_bins_group(const VcbArgs *__restrict__ args, GroupQueue q)
{
    __shared__ int s_item;
    gq_run(q, &s_item, [&](int m, int vb, int) {
        const VcbArgs a = args[m];
        vcross_bins_block<P, LMAX>(a, vb);
        return true;
    });
}

// total potential per point: own cell (FP64) plus the pair contributions in
// atom order, summed with TwoSum; writes V and cj = w V / 2
__global__ void k_vcross_gather(size_t npts, size_t npad, int natoms, int cell0, int nrad, int nang,
                                const int *__restrict__ pos, const float2 *__restrict__ pairv,
                                const double *__restrict__ Vown, const double *__restrict__ W,
                                double *__restrict__ V, double *__restrict__ cj, float *__restrict__ cj32)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    if (p >= npts) { V[p] = 0.0; cj[p] = 0.0; cj32[p] = 0.f; return; }
    const int a = cell0 + (int)(p / ((size_t)nrad * nang));
    float vh = 0.f, vl = 0.f;
    for (int k = 0; k < natoms; ++k) {
        if (k == a) continue;
        const float2 v = pairv[pos[p * natoms + k]];
        two_sum_acc(vh, vl, v.x);
        vl += v.y;
    }
    const double Vt = Vown[p] + ((double)vh + (double)vl);
    V[p] = Vt;
    const double c = 0.5 * (W[p] * Vt);
    cj[p] = c;
    cj32[p] = (float)c;
}

// K5c+K5e+E_J (mixed, one launch): the own-cell potential
// V_own = (1 / r) sum_lm U_lm(r_i) Y_lm(j) in double-float with exact products,
// plus the pair contributions in atom order summed with TwoSum; writes V and
// cj = w V / 2, and sums E_J = sum_p cj rho_raw (block partials, the last block
// adds them in order).  A block takes one cell, a slab of kGoSlab antipodal
// pairs of Lebedev directions and kGoShells radial shells: the Y_lm (hi, lo) of
// the slab's first directions are staged in shared memory once, a warp takes a
// shell at a time with a lane per pair, and the shell's U_lm row is one
// broadcast load per (l, m).  Since Y_lm(-r) = (-1)^l Y_lm(r), a lane sums the
// even-l and the odd-l terms once and has V_own at both points of its pair
// (even + odd, even - odd): half the products of a lane per direction.
constexpr int kGoSlab = 32;
constexpr int kGoShells = 8;
constexpr int kGoThreads = 256;

__device__ __forceinline__ void gather_own_block(const GoArgs A, int b, int nblk)
{
    const size_t npts = A.npts, npad = A.npad, uhalf = A.uhalf;
    const int natoms = A.natoms, cell0 = A.cell0, nrad = A.nrad, nang = A.nang, nlm = A.nlm;
    const int nslab = A.nslab, nsplit = A.nsplit, scaled = A.scaled;
    const int *__restrict__ pos = A.pos;
    const float2 *__restrict__ pairv = A.pairv;
    const float *__restrict__ U32T = A.U32T, *__restrict__ Y32 = A.Y32;
    const double *__restrict__ invr = A.invr, *__restrict__ W = A.W, *__restrict__ rho = A.rho;
    double *__restrict__ V = A.V, *__restrict__ cj = A.cj;
    float *__restrict__ cj32 = A.cj32;
    double *__restrict__ part = A.part;
    double *scal = A.scal;
    int *counter = A.counter;
    const int npair = A.npair;
    const int2 *__restrict__ pairs = A.pairs;
    extern __shared__ float go_smem[];                       // [2][nlm][kGoSlab] Y_lm, [2][kGoShells][nlm] U_lm
    __shared__ double sh[32];
    __shared__ int s_last;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int al = b / (nslab * nsplit), rest = b % (nslab * nsplit), slab = rest / nsplit, sp = rest % nsplit;
    const int a = cell0 + al, k0 = slab * kGoSlab;          // the slab's first antipodal pair
    const int i_beg = sp * kGoShells, i_end = min(nrad, i_beg + kGoShells);
    float *syh = go_smem, *syl = go_smem + (size_t)nlm * kGoSlab;
    float *suh = syl + (size_t)nlm * kGoSlab, *sul = suh + (size_t)kGoShells * nlm;
    // Y_lm at the first direction of each of the slab's pairs (Y_lm at the
    // antipode is (-1)^l times it)
    for (int e = tid; e < nlm * kGoSlab; e += kGoThreads) {
        const int lm = e / kGoSlab, k = k0 + e % kGoSlab;
        const int j = k < npair ? __ldg(&pairs[k].x) : 0;
        syh[e] = k < npair ? Y32[(size_t)lm * nang + j] : 0.f;
        syl[e] = k < npair ? Y32[(size_t)nlm * nang + (size_t)lm * nang + j] : 0.f;
    }
    // the block's shells of U_lm (rows (a, i) of the transposed split table are contiguous)
    {
        const size_t u0 = ((size_t)a * nrad + i_beg) * nlm;
        const int nu = (i_end - i_beg) * nlm;
        for (int e = tid; e < nu; e += kGoThreads) {
            suh[e] = U32T[u0 + e];
            sul[e] = U32T[uhalf + u0 + e];
        }
    }
    if (b == 0)                                              // the padded tail of the point arrays
        for (size_t p = npts + tid; p < npad; p += kGoThreads) {
            V[p] = 0.0;
            cj[p] = 0.0;
            cj32[p] = 0.f;
        }
    __syncthreads();
    const int k = k0 + lane;
    const int2 ja = k < npair ? __ldg(&pairs[k]) : make_int2(0, 0);
    const int lmax = (int)sqrtf((float)nlm + 0.5f) - 1;
    double ej = 0.0;
    for (int i = i_beg + warp; i < i_end; i += kGoThreads / 32) {
        const float *uh = suh + (size_t)(i - i_beg) * nlm, *ul = sul + (size_t)(i - i_beg) * nlm;
        // even-l and odd-l parts of the own-cell sum, two accumulators each
        float s0 = 0.f, e0 = 0.f, s1 = 0.f, e1 = 0.f, s2 = 0.f, e2 = 0.f, s3 = 0.f, e3 = 0.f;
        for (int l = 0; l <= lmax; ++l) {
            int lm = l * l;
            const int lm1 = lm + 2 * l + 1;
            if (l & 1) {
                for (; lm + 1 < lm1; lm += 2) {
                    df_mac(s2, e2, uh[lm], ul[lm], syh[lm * kGoSlab + lane], syl[lm * kGoSlab + lane]);
                    df_mac(s3, e3, uh[lm + 1], ul[lm + 1], syh[(lm + 1) * kGoSlab + lane], syl[(lm + 1) * kGoSlab + lane]);
                }
                if (lm < lm1) df_mac(s2, e2, uh[lm], ul[lm], syh[lm * kGoSlab + lane], syl[lm * kGoSlab + lane]);
            } else {
                for (; lm + 1 < lm1; lm += 2) {
                    df_mac(s0, e0, uh[lm], ul[lm], syh[lm * kGoSlab + lane], syl[lm * kGoSlab + lane]);
                    df_mac(s1, e1, uh[lm + 1], ul[lm + 1], syh[(lm + 1) * kGoSlab + lane], syl[(lm + 1) * kGoSlab + lane]);
                }
                if (lm < lm1) df_mac(s0, e0, uh[lm], ul[lm], syh[lm * kGoSlab + lane], syl[lm * kGoSlab + lane]);
            }
        }
        float cbound[2] = {0.f, 0.f};      // |cj32 / w| of the pair's points (chunk bounds)
        int cchunk[2] = {-1, -1};
        if (k < npair) {
            const dfl ev = df_add(df_norm(s0, e0), df_norm(s1, e1)), od = df_add(df_norm(s2, e2), df_norm(s3, e3));
            // the pair's two points: V_own = even + odd at j, even - odd at its antipode
#pragma unroll
            for (int t = 0; t < 2; ++t) {
                const size_t p = ((size_t)al * nrad + i) * nang + (t ? ja.y : ja.x);
                const dfl vs = t ? df_sub(ev, od) : df_add(ev, od);
                const double vown = df_to(vs) * invr[p];
                float vh = 0.f, vl = 0.f;
                const int *pp = pos + p * natoms;
                // eight atoms at a time: their places, then their contributions, then
                // the sum in atom order
                for (int q0 = 0; q0 < natoms; q0 += 8) {
                    int q[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) q[u] = (q0 + u < natoms && q0 + u != a) ? pp[q0 + u] : -1;
                    float2 v[8];
#pragma unroll
                    for (int u = 0; u < 8; ++u) v[u] = q[u] >= 0 ? pairv[q[u]] : make_float2(0.f, 0.f);
#pragma unroll
                    for (int u = 0; u < 8; ++u)
                        if (q[u] >= 0) {
                            two_sum_acc(vh, vl, v[u].x);
                            vl += v[u].y;
                        }
                }
                const double Vt = vown + ((double)vh + (double)vl);
                V[p] = Vt;
                const double c = 0.5 * (W[p] * Vt);
                cj[p] = c;
                const float cf = (float)c;
                cj32[p] = cf;
                if (A.cmax) {
                    cbound[t] = fabsf(cf) * A.winv[p];
                    cchunk[t] = (int)(p / A.chunk_pts);
                }
                ej += c * rho[p];
            }
        }
        if (A.cmax) {                       // every lane of the warp, valid pair or not
            warp_chunk_max(A.cmax, cchunk[0], cbound[0]);
            warp_chunk_max(A.cmax, cchunk[1], cbound[1]);
        }
    }
    ej = block_sum(ej, sh);
    if (tid == 0) part[b] = ej;
    if (!last_block_of(counter, nblk, &s_last)) return;
    double t = 0.0;
    for (int k = tid; k < nblk; k += kGoThreads) t += __ldcg(part + k);
    t = block_sum(t, sh);
    if (tid == 0) scal[kScalEJ] = scaled ? t / __ldcg(scal + kScalScale) : t;
}

__global__ void __launch_bounds__(kGoThreads) k_vcross_gather_own(const GoArgs a)
{
    pdl_wait();
    gather_own_block(a, (int)blockIdx.x, (int)gridDim.x);
    pdl_signal();
}

__global__ void __launch_bounds__(kGoThreads) k_vcross_gather_own_group(const GoArgs *__restrict__ args, GroupQueue q)
{
    __shared__ int s_item;
    gq_run(q, &s_item, [&](int m, int vb, int nvb) {
        const GoArgs a = args[m];
        gather_own_block(a, vb, nvb);
        return true;
    });
}

// Order the (point, other atom) pairs by (atom, spline interval of their
// distance), stably in the enumeration order (point, then atom): pos[p][k] is
// the place of pair (p, k).  On the device: the pairs' keys (FP64 distance,
// the interval rule of spline_interval(): clamp below the first and beyond the
// last knot) and a histogram of the keys, a stable radix sort of the keys with
// the enumeration index as payload, then the per-pair geometry at its sorted
// place.  The runs of at most kCrossTask pairs inside one bin (the tasks of
// k_vcross_bins) are formed on the host from the bin counts.
__device__ __forceinline__ void pair_of_enum(size_t e, int na, int cell0, int per_atom, size_t &p, int &k)
{
    p = e / (size_t)(na - 1);
    const int j = (int)(e - p * (size_t)(na - 1));
    const int a = cell0 + (int)(p / per_atom);
    k = j < a ? j : j + 1;          // every atom but the point's own
}

__device__ __forceinline__ void pair_interval(double r, const double *__restrict__ sx, int N, int &iv, double &t)
{
    if (r < sx[0]) { iv = 0; t = 0.0; return; }
    if (r >= sx[N - 1]) { iv = N - 1; t = 0.0; return; }
    int lo = 0, hi = N;                 // first i with sx[i] >= r
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (sx[mid] < r) lo = mid + 1;
        else hi = mid;
    }
    const int i = max(1, min(N - 1, lo));
    iv = i - 1;
    t = r - sx[iv];
}

__global__ void k_pair_keys(size_t npairs, int na, int cell0, int per_atom, int N, const double *__restrict__ X,
                            const double *__restrict__ Y, const double *__restrict__ Z,
                            const double *__restrict__ atoms, const double *__restrict__ sx, int *__restrict__ key,
                            int *__restrict__ idx, unsigned *__restrict__ count)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= npairs) return;
    size_t p;
    int k;
    pair_of_enum(e, na, cell0, per_atom, p, k);
    const double dx = X[p] - atoms[4 * k], dy = Y[p] - atoms[4 * k + 1], dz = Z[p] - atoms[4 * k + 2];
    int iv;
    double t;
    pair_interval(sqrt(dx * dx + dy * dy + dz * dz), sx, N, iv, t);
    const int kk = k * N + iv;
    key[e] = kk;
    idx[e] = (int)e;
    atomicAdd(count + kk, 1u);
}

__global__ void k_pair_place(size_t npairs, int na, int cell0, int per_atom, int N, const double *__restrict__ X,
                             const double *__restrict__ Y, const double *__restrict__ Z,
                             const double *__restrict__ atoms, const double *__restrict__ sx,
                             const int *__restrict__ order, float4 *__restrict__ geo, float2 *__restrict__ tk,
                             int *__restrict__ pos)
{
    const size_t dst = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (dst >= npairs) return;
    const size_t e = (size_t)order[dst];
    size_t p;
    int k;
    pair_of_enum(e, na, cell0, per_atom, p, k);
    // the geometry of a pair is fixed for the grid: direction, 1/r and the
    // spline offset are formed in FP64 and rounded once to FP32
    const double dx = X[p] - atoms[4 * k], dy = Y[p] - atoms[4 * k + 1], dz = Z[p] - atoms[4 * k + 2];
    const double r = sqrt(dx * dx + dy * dy + dz * dz);
    int iv;
    double t;
    pair_interval(r, sx, N, iv, t);
    geo[dst] = make_float4((float)(dx / r), (float)(dy / r), (float)(dz / r), (float)(1.0 / r));
    const uint32_t kv = ((uint32_t)k << 16) | (uint32_t)iv;
    tk[dst] = make_float2((float)t, __uint_as_float(kv));
    pos[p * na + k] = (int)dst;
}

int cross_pairs_setup(dftg_ctx *c)
{
    const size_t n = c->npts;
    const int na = c->natoms, N = c->nrad, per_atom = c->nrad * c->nang;
    if (na < 2) { c->npairs = 0; return DFTG_OK; }
    const size_t npairs = n * (size_t)(na - 1);
    if (npairs > (size_t)INT32_MAX) { set_error("too many (point, atom) pairs: %zu", npairs); return DFTG_ERR_ARG; }
    const int nkeys = na * N;
    int bits = 1;
    while ((1 << bits) < nkeys) ++bits;
    // device work arrays: keys and indices in and out, the histogram, the sorter's scratch
    int *kin = nullptr, *iin = nullptr, *kout = nullptr, *iout = nullptr;
    unsigned *cnt = nullptr;
    double *sx = nullptr;
    void *tmp = nullptr;
    size_t tmp_bytes = 0;
    cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, kin, kout, iin, iout, (int)npairs, 0, bits, c->stream);
    const size_t ibytes = sizeof(int) * npairs;
    char *work = nullptr;
    const size_t wbytes = 4 * ibytes + sizeof(unsigned) * nkeys + sizeof(double) * N + tmp_bytes + 256;
    DFTG_CUDA(cudaMalloc(&work, wbytes));
    kin = reinterpret_cast<int *>(work);
    iin = kin + npairs;
    kout = iin + npairs;
    iout = kout + npairs;
    cnt = reinterpret_cast<unsigned *>(iout + npairs);
    sx = reinterpret_cast<double *>((reinterpret_cast<uintptr_t>(cnt + nkeys) + 15) & ~(uintptr_t)15);
    tmp = reinterpret_cast<void *>((reinterpret_cast<uintptr_t>(sx + N) + 127) & ~(uintptr_t)127);
    int rc = DFTG_OK;
    std::vector<double> sxh(N);
    for (int i = 0; i < N; ++i) sxh[i] = c->r_n[N - 1 - i];   // increasing spline abscissae
    std::vector<unsigned> count(nkeys);
    cudaError_t e = cudaMemcpyAsync(sx, sxh.data(), sizeof(double) * N, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(cnt, 0, sizeof(unsigned) * nkeys, c->stream);
    const unsigned nb = (unsigned)((npairs + 255) / 256);
    if (e == cudaSuccess) {
        k_pair_keys<<<nb, 256, 0, c->stream>>>(npairs, na, c->cell0, per_atom, N, c->d_x, c->d_y, c->d_z, c->d_atoms, sx, kin,
                                              iin, cnt);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess)
        e = cub::DeviceRadixSort::SortPairs(tmp, tmp_bytes, kin, kout, iin, iout, (int)npairs, 0, bits, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(count.data(), cnt, sizeof(unsigned) * nkeys, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess && !c->d_pairs) e = cudaMalloc(&c->d_pairs, (sizeof(float4) + sizeof(float2)) * npairs);
    if (e == cudaSuccess && !c->d_pairpos) e = cudaMalloc(&c->d_pairpos, sizeof(int) * n * (size_t)na);
    if (e == cudaSuccess && !c->d_pairv) e = cudaMalloc(&c->d_pairv, sizeof(float2) * npairs);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_pairpos, 0, sizeof(int) * n * (size_t)na, c->stream);
    if (e == cudaSuccess) {
        char *base = static_cast<char *>(c->d_pairs);
        k_pair_place<<<nb, 256, 0, c->stream>>>(npairs, na, c->cell0, per_atom, N, c->d_x, c->d_y, c->d_z, c->d_atoms, sx, iout,
                                               reinterpret_cast<float4 *>(base),
                                               reinterpret_cast<float2 *>(base + sizeof(float4) * npairs),
                                               c->d_pairpos);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "cross-atom pair sort", __FILE__, __LINE__);
    cudaFree(work);
    if (rc != DFTG_OK) return rc;
    // tasks: runs of at most kCrossTask pairs inside one bin, bins in key order
    std::vector<int4> tasks;
    size_t start = 0;
    for (int kk = 0; kk < nkeys; ++kk) {
        const size_t cn = count[kk];
        for (size_t o = 0; o < cn; o += kCrossTask)
            tasks.push_back(make_int4((int)(start + o), (int)std::min<size_t>(kCrossTask, cn - o), kk / N, kk % N));
        start += cn;
    }
    c->npairs = npairs;
    c->ncross_tasks = (int)tasks.size();
    DFTG_CUDA(cudaMalloc(&c->d_cross_tasks, sizeof(int4) * tasks.size()));
    DFTG_CUDA(cudaMemcpy(c->d_cross_tasks, tasks.data(), sizeof(int4) * tasks.size(), cudaMemcpyHostToDevice));
    return DFTG_OK;
}

// E_J = 2 tr(P J) = sum_p (w V / 2) rho_raw (the J assembly contracted with P,
// evaluated directly on the grid in FP64): deterministic block partials, summed
// by the last block
__global__ void __launch_bounds__(256) k_ej(size_t npad, const double *__restrict__ cj, const double *__restrict__ rho,
                                            double *__restrict__ part, int scaled, double *scal, int *counter)
{
    __shared__ double sh[32];
    __shared__ int s_last;
    double v = 0.0;   // grid-stride: a few points per thread, one block sum per block
    for (size_t p = (size_t)blockIdx.x * 256 + threadIdx.x; p < npad; p += (size_t)gridDim.x * 256) v += cj[p] * rho[p];
    v = block_sum(v, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = v;
    if (!last_block(counter, &s_last)) return;
    // last block: sum of the block partials in a fixed order; rho on the device
    // carries the correction factor when scaled
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += 256) t += __ldcg(part + i);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) scal[kScalEJ] = scaled ? t / scal[kScalScale] : t;
}

StepLaunch<VcbArgs> step_vcross_bins(const dftg_ctx *c)
{
    StepLaunch<VcbArgs> s;
    s.args = VcbArgs{c->nrad, c->lmax, reinterpret_cast<const int4 *>(c->d_cross_tasks),
                     reinterpret_cast<const float4 *>(c->d_pairs),
                     reinterpret_cast<const float2 *>(static_cast<const char *>(c->d_pairs) + sizeof(float4) * c->npairs),
                     c->d_splm, reinterpret_cast<float2 *>(c->d_pairv)};
    s.blocks = c->npairs > 0 ? (int)c->ncross_tasks : 0;
    s.smem = sizeof(float4) * 2 * c->nlm;
    return s;
}

// the kernel variant of an lmax: fully unrolled for the grid presets' cut-offs
template <int LMAX>
struct VcbSingle {
    static cudaError_t run(const StepLaunch<VcbArgs> &s, cudaStream_t st)
    {
        return launch_pdl(k_vcross_bins<kCrossPerThread, LMAX>, s.blocks, 128, s.smem, st, s.args);
    }
};
template <int LMAX>
struct VcbGroup {
    static int run(const VcbArgs *d, const GroupQueue &q, size_t smem, int nsm, cudaStream_t st)
    {
        int occ = 0;
        DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_vcross_bins_group<kCrossPerThread, LMAX>, 128, smem));
        const int grid = group_grid(q, occ, nsm);
        if (grid > 0) k_vcross_bins_group<kCrossPerThread, LMAX><<<grid, 128, smem, st>>>(d, q);
        return DFTG_OK;
    }
};

static int launch_vcross_bins(dftg_ctx *c)
{
    const StepLaunch<VcbArgs> s = step_vcross_bins(c);
    switch (c->lmax) {
    case 5: DFTG_CUDA(VcbSingle<5>::run(s, c->stream)); break;
    case 6: DFTG_CUDA(VcbSingle<6>::run(s, c->stream)); break;
    case 8: DFTG_CUDA(VcbSingle<8>::run(s, c->stream)); break;
    case 10: DFTG_CUDA(VcbSingle<10>::run(s, c->stream)); break;
    case 11: DFTG_CUDA(VcbSingle<11>::run(s, c->stream)); break;
    default: DFTG_CUDA(VcbSingle<-1>::run(s, c->stream)); break;
    }
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// lmax: the molecules' common cut-off (the unrolled variant), or -1 when they differ
int group_vcross_bins(const VcbArgs *d_args, const GroupQueue &q, int lmax, size_t smem, int nsm, cudaStream_t st)
{
    int rc = DFTG_OK;
    switch (lmax) {
    case 5: rc = VcbGroup<5>::run(d_args, q, smem, nsm, st); break;
    case 6: rc = VcbGroup<6>::run(d_args, q, smem, nsm, st); break;
    case 8: rc = VcbGroup<8>::run(d_args, q, smem, nsm, st); break;
    case 10: rc = VcbGroup<10>::run(d_args, q, smem, nsm, st); break;
    case 11: rc = VcbGroup<11>::run(d_args, q, smem, nsm, st); break;
    default: rc = VcbGroup<-1>::run(d_args, q, smem, nsm, st); break;
    }
    if (rc != DFTG_OK) return rc;
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

StepLaunch<MpArgs> step_multipole(const dftg_ctx *c, bool rw_ready)
{
    int ngroup = 0;                          // groups of at most kMpLG rows of one degree l
    for (int l = 0; l <= c->lmax; ++l) ngroup += (2 * l + 1 + kMpLG - 1) / kMpLG;
    StepLaunch<MpArgs> s;
    s.args = MpArgs{c->natoms, c->cell0, c->nrad, c->nang, c->lmax, ngroup, (c->prec_mask & kPrecCross) ? 0 : 1,
                    rw_ready ? c->d_rw32 : nullptr, c->npad, c->d_rho, c->d_wb, c->d_w, c->d_Ywt32, c->d_maps32,
                    c->d_scal, c->d_U, c->d_U32, c->d_U32T, c->d_spl, c->d_splm, c->d_lebpair, c->nlebpair};
    s.blocks = c->ncell * ngroup;
    s.smem = multipole_smem(c->nrad, c->nang);
    return s;
}

int group_multipole(const MpArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st)
{
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_multipole_group), device));
    int occ = 0;
    DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_multipole_group, kMpThreads, smem));
    const int grid = group_grid(q, occ, nsm);
    if (grid > 0) k_multipole_group<<<grid, kMpThreads, smem, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// multipole part of the Hartree step for the context's cells (atoms cell0 ..
// cell0 + ncell - 1, whose points the context holds): rho_lm, the radial
// Poisson maps, the own-cell potential and the spline coefficients of U_lm
int launch_hartree_multipoles(dftg_ctx *c)
{
    const int N = c->nrad, nlm = c->nlm, nc = c->ncell, c0 = c->cell0;
    // the mixed multipole kernels keep radial vectors per block in shared
    // memory: up to 256 radial points (the FP64 kernels take any)
    const bool mp = (c->prec_mask & kPrecMultipole) != 0 && N <= 256 && c->nlebpair > 0;
    const size_t rplane = (size_t)c->natoms * nlm * N;
    const int nrhs = nc * nlm;
    if (mp) {
        // rho_lm, Poisson and splines in one launch per (cell, group of l, m rows)
        const StepLaunch<MpArgs> st = step_multipole(c, c->rw_ready);
        if (st.smem > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_multipole), c->device));
        DFTG_CUDA(launch_pdl(k_multipole, st.blocks, kMpThreads, st.smem, c->stream, st.args));
        DFTG_MARK(c, "multipole");
        if (!(c->prec_mask & kPrecCross)) {
            // the FP64 cross-atom step takes the own-cell potential from memory:
            // a double-float GEMM [(a, i) x lm] x [lm x j]
            const int M = nc * N;
            const size_t off = (size_t)c0 * N * nlm;
            dim3 grid((unsigned)((c->nang + kDgBN - 1) / kDgBN), (unsigned)((M + kDgBM - 1) / kDgBM), 1);
            k_dfgemm<EpiVown><<<grid, 128, 0, c->stream>>>(M, c->nang, nlm, c->d_U32T + off, c->d_U32T + rplane + off,
                                                           nlm, c->d_Y32, c->d_Y32 + (size_t)nlm * c->nang, c->nang,
                                                           EpiVown{c->nang, c->d_invr, c->d_Vown});
            DFTG_LAUNCH_CHECK();
            DFTG_MARK(c, "vown");
        }
        return DFTG_OK;
    }
    k_rholm<<<nc * N, 96, sizeof(double) * c->nang, c->stream>>>(N, c->nang, nlm, c0, c->d_rho, c->d_wb, c->d_Yw,
                                                                c->d_rholm);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "rholm");
    k_poisson<<<nrhs, 128, sizeof(double) * N, c->stream>>>(c->natoms, c0, N, c->lmax, c->d_Gt, c->d_Gb, c->d_rholm,
                                                            c->d_scal, c->d_U, c->d_U32);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "poisson");
    const unsigned npb = (unsigned)((c->npts + 127) / 128);
    k_vown<<<npb, 128, 0, c->stream>>>(c->npts, N, c->nang, nlm, c0, c->d_rn, c->d_leb, c->d_Y, c->d_U, c->d_Vown);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "vown");
    k_splines<<<nrhs, 128, sizeof(double) * 2 * N, c->stream>>>(c->natoms, c0, N, nlm, c->d_splf, c->d_Kt, c->d_U,
                                                                c->d_fold, c->d_spl, c->d_splm);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "splines");
    return DFTG_OK;
}

StepLaunch<GoArgs> step_gather_own(const dftg_ctx *c, bool rho_scaled)
{
    const int N = c->nrad;
    const int nslab = (c->nlebpair + kGoSlab - 1) / kGoSlab, nsplit = (N + kGoShells - 1) / kGoShells;
    StepLaunch<GoArgs> s;
    s.args = GoArgs{c->npts, c->npad, (size_t)c->natoms * c->nlm * N, c->natoms, c->cell0, N, c->nang, c->nlm, nslab,
                    nsplit, rho_scaled ? 1 : 0, c->d_pairpos, reinterpret_cast<const float2 *>(c->d_pairv), c->d_U32T,
                    c->d_Y32, c->d_invr, c->d_w, c->d_rho, c->d_V, c->d_cj, c->d_cj32, c->d_red, c->d_scal,
                    c->d_counters + kCntEJ, c->d_lebpair, c->nlebpair,
                    cmax_route(c) ? c->d_ct_cmax + c->ct_nchunk : nullptr, c->d_ct_winv, c->ct_kbpc * 32};
    s.blocks = c->ncell * nslab * nsplit;
    s.smem = sizeof(float) * 2 * (size_t)c->nlm * (kGoSlab + kGoShells);
    return s;
}

int group_gather_own(const GoArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st)
{
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_vcross_gather_own_group), device));
    int occ = 0;
    DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_vcross_gather_own_group, kGoThreads, smem));
    const int grid = group_grid(q, occ, nsm);
    if (grid > 0) k_vcross_gather_own_group<<<grid, kGoThreads, smem, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// cross-atom part: the potential of every other atom's spline expansion on the
// context's points, the total V, cj = w V / 2 and E_J
int launch_hartree_cross(dftg_ctx *c)
{
    const int N = c->nrad;
    const bool mp = (c->prec_mask & kPrecMultipole) != 0 && N <= 256 && c->nlebpair > 0;
    const unsigned nb = (unsigned)(c->npad / 128);
    if (c->prec_mask & kPrecCross) {
        if (c->npairs > 0) {
            DFTG_TRY_L(launch_vcross_bins(c));
            DFTG_MARK(c, "vcross_bins");
        }
        if (mp) {
            // own-cell potential, total potential and E_J in one pass
            const StepLaunch<GoArgs> st = step_gather_own(c, c->rho_scaled);
            if ((size_t)st.blocks > c->red_elems) { set_error("reduction buffer too small for %d blocks", st.blocks); return DFTG_ERR_STATE; }
            if (st.smem > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_vcross_gather_own), c->device));
            DFTG_CUDA(launch_pdl(k_vcross_gather_own, st.blocks, kGoThreads, st.smem, c->stream, st.args));
            DFTG_MARK(c, "vcross");
            return DFTG_OK;
        }
        k_vcross_gather<<<(unsigned)((c->npad + 127) / 128), 128, 0, c->stream>>>(
            c->npts, c->npad, c->natoms, c->cell0, N, c->nang, c->d_pairpos, reinterpret_cast<const float2 *>(c->d_pairv),
            c->d_Vown, c->d_w, c->d_V, c->d_cj, c->d_cj32);
    } else
        k_vcross64<<<nb, 128, 0, c->stream>>>(c->npts, c->npad, c->natoms, c->cell0, N, c->nang, c->lmax, c->d_atoms,
                                              c->d_x, c->d_y, c->d_z, c->d_w, c->d_sx, c->d_spl, c->d_pre, c->d_rec,
                                              c->d_Vown, c->d_V, c->d_cj, c->d_cj32);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "vcross");
    const unsigned ne = (unsigned)std::min<size_t>((c->npad + 255) / 256, 2 * 152);
    k_ej<<<ne, 256, 0, c->stream>>>(c->npad, c->d_cj, c->d_rho, c->d_red, c->rho_scaled ? 1 : 0, c->d_scal,
                                    c->d_counters + kCntEJ);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "hartree_energy");
    return DFTG_OK;
}

int launch_hartree(dftg_ctx *c)
{
    DFTG_TRY_L(launch_hartree_multipoles(c));
    return launch_hartree_cross(c);
}

}  // namespace dftg
