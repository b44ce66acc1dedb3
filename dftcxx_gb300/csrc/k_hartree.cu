// k_hartree.cu -- Becke-Poisson Hartree potential (MolecularGrid::calculate_hartree_potential,
// moleculargrid.cpp:336-389, and AtomicGrid::calculate_rho_lm / calculate_U_lm,
// atomicgrid.cpp:241-466).
//
// K5a rho_lm[a][lm][i] = 4 pi sum_j rho w_becke w_leb,j Y_lm(dir_j): one CTA per
//     (atom, radial shell); Y_lm of the Lebedev directions precomputed once.
// K5b radial Poisson solve per (atom, lm): the finite-difference operator
//     depends only on (nrad, l), so it is LU-factored once per l on the host
//     (partial pivoting, same elimination order as the reference's dense LU)
//     and every right-hand side is swept on the device.
// K5c own-cell potential V_n(p) = sum_lm U_lm(r_i) / r Y_lm (atomicgrid.cpp:439-462).
// K5d cubic splines of U_lm over increasing r (cspline.cpp:66-142), one thread
//     per (atom, lm), stored [atom][lm][interval][4] (interval nrad-1 holds the
//     clamp value of the last knot).
// K5e cross-atom potential: for every point and every other atom k,
//     sum_lm U^k_lm(r)/r Y_lm with Y_lm by Cartesian recursion (no atan2/acos)
//     and an O(1) spline-interval lookup from the analytic radial map
//     r = (1+x)/(1-x), x = cos(pi p/(N+1)) (moleculargrid.cpp:342-380).
//     T = double (FP64 path) or float (mixed path); V accumulates in FP64.
#include <cmath>
#include <vector>
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

int hartree_setup(dftg_ctx *c)
{
    const int nang = c->nang, nlm = c->nlm, N = c->nrad, S = N + 2;
    std::vector<double> Y((size_t)nlm * nang), Yw((size_t)nlm * nang), pre(nlm);
    std::vector<double> leb((size_t)nang * 4);
    DFTG_CUDA(cudaMemcpy(leb.data(), c->d_leb, sizeof(double) * nang * 4, cudaMemcpyDeviceToHost));
    for (int l = 0; l <= c->lmax; ++l)
        for (int m = -l; m <= l; ++m) {
            int lm = l * l + l + m;
            pre[lm] = sh_prefactor(l, m);
            for (int j = 0; j < nang; ++j) {
                double y = ylm_host(l, m, leb[4 * j], leb[4 * j + 1], leb[4 * j + 2]);
                Y[(size_t)lm * nang + j] = y;
                Yw[(size_t)lm * nang + j] = y * leb[4 * j + 3];
            }
        }
    std::vector<double> A((size_t)S * S), LU((size_t)(c->lmax + 1) * S * S);
    std::vector<int> piv((size_t)(c->lmax + 1) * S);
    poisson_matrix(N, c->r_n.data(), A.data());
    for (int l = 0; l <= c->lmax; ++l) {
        double *M = LU.data() + (size_t)l * S * S;
        for (size_t t = 0; t < (size_t)S * S; ++t) M[t] = A[t];
        for (int i = 1; i < N + 1; ++i)
            M[(size_t)i * S + i] -= (double)l * (double)(l + 1) / (c->r_n[i - 1] * c->r_n[i - 1]);
        lu_factor(S, M, piv.data() + (size_t)l * S);
    }
    std::vector<double> rec((size_t)2 * nlm, 0.0);
    for (int l = 0; l <= c->lmax; ++l)
        for (int m = 0; m < l; ++m) {
            rec[2 * (l * l + l + m)] = (double)(2 * l - 1) / (double)(l - m);
            rec[2 * (l * l + l + m) + 1] = (double)(l + m - 1) / (double)(l - m);
        }
    std::vector<float> pre32(pre.begin(), pre.end()), rec32(rec.begin(), rec.end());
    DFTG_CUDA(cudaMemcpy(c->d_rec, rec.data(), sizeof(double) * rec.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_rec32, rec32.data(), sizeof(float) * rec32.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_pre32, pre32.data(), sizeof(float) * pre32.size(), cudaMemcpyHostToDevice));
    std::vector<double> sx(N);
    for (int i = 0; i < N; ++i) sx[i] = c->r_n[N - 1 - i];
    DFTG_CUDA(cudaMemcpy(c->d_Y, Y.data(), sizeof(double) * Y.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_Yw, Yw.data(), sizeof(double) * Yw.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_pre, pre.data(), sizeof(double) * pre.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_LU, LU.data(), sizeof(double) * LU.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_piv, piv.data(), sizeof(int) * piv.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_sx, sx.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    return DFTG_OK;
}

// ------------------------------------------------------------------ kernels

// K5a: CTA per (atom, shell)
__global__ void k_rholm(int nrad, int nang, int nlm, const double *__restrict__ rho, const double *__restrict__ wb,
                        const double *__restrict__ Yw, double *__restrict__ rholm)
{
    extern __shared__ double s_rw[];   // [nang]
    const int a = blockIdx.x / nrad, i = blockIdx.x % nrad;
    const size_t base = ((size_t)a * nrad + i) * nang;
    for (int j = threadIdx.x; j < nang; j += blockDim.x) s_rw[j] = rho[base + j] * wb[base + j];
    __syncthreads();
    for (int lm = threadIdx.x; lm < nlm; lm += blockDim.x) {
        const double *y = Yw + (size_t)lm * nang;
        double s = 0.0;
        for (int j = 0; j < nang; ++j) s += s_rw[j] * y[j];
        rholm[((size_t)a * nlm + lm) * nrad + i] = s * 4.0 * kPi;
    }
}

// K5b: one thread per (atom, lm); g in shared memory [S][32]
__global__ void k_poisson(int natoms, int nrad, int lmax, const double *__restrict__ rn,
                          const double *__restrict__ LU, const int *__restrict__ piv,
                          const double *__restrict__ rholm, const double *__restrict__ scal,
                          double *__restrict__ U)
{
    extern __shared__ double s_g[];
    const int nlm = (lmax + 1) * (lmax + 1);
    const int t = threadIdx.x;
    const int id = blockIdx.x * 32 + t;
    const int N = nrad, S = N + 2;
    if (id >= natoms * nlm) return;
    const int a = id / nlm, lm = id % nlm;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) ++l;
    const double *F = LU + (size_t)l * S * S;
    const int *pv = piv + (size_t)l * S;
    const double *R = rholm + ((size_t)a * nlm + lm) * N;
    double *g = s_g;   // g[i*32 + t]
    g[t] = (lm == 0) ? sqrt(4.0 * kPi) * scal[kScalAtomQ + a] : 0.0;
    for (int i = 1; i < N + 1; ++i) g[i * 32 + t] = -4.0 * kPi * rn[i - 1] * R[i - 1];
    g[(N + 1) * 32 + t] = 0.0;
    // the factor rows were exchanged whole (multipliers included), so the
    // interchanges are applied to g first, then the unit-lower sweep
    for (int k = 0; k < S; ++k) {
        const int p = pv[k];
        if (p != k) { double tmp = g[k * 32 + t]; g[k * 32 + t] = g[p * 32 + t]; g[p * 32 + t] = tmp; }
    }
    for (int k = 0; k < S; ++k) {
        const double gk = g[k * 32 + t];
        for (int i = k + 1; i < S; ++i) {
            const double f = F[(size_t)i * S + k];
            if (f != 0.0) g[i * 32 + t] -= f * gk;
        }
    }
    for (int i = S - 1; i >= 0; --i) {
        double s = g[i * 32 + t];
        for (int j = i + 1; j < S; ++j) s -= F[(size_t)i * S + j] * g[j * 32 + t];
        g[i * 32 + t] = s / F[(size_t)i * S + i];
    }
    double *u = U + ((size_t)a * nlm + lm) * N;
    for (int i = 1; i < N + 1; ++i) u[i - 1] = g[i * 32 + t];
}

// K5c: own-cell potential for every point
__global__ void k_vown(size_t npts, int nrad, int nang, int nlm, const double *__restrict__ rn,
                       const double *__restrict__ leb, const double *__restrict__ Y, const double *__restrict__ U,
                       double *__restrict__ Vown)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int per_atom = nrad * nang;
    const int a = (int)(p / per_atom), rem = (int)(p % per_atom), i = rem / nang, j = rem % nang;
    const double ri = rn[i];
    const double px = leb[4 * j] * ri, py = leb[4 * j + 1] * ri, pz = leb[4 * j + 2] * ri;
    const double inv_r = 1.0 / sqrt(px * px + py * py + pz * pz);
    const double *u = U + (size_t)a * nlm * nrad + i;
    double v = 0.0;
    for (int lm = 0; lm < nlm; ++lm) v += inv_r * Y[(size_t)lm * nang + j] * u[(size_t)lm * nrad];
    Vown[p] = v;
}

// K5d: spline coefficients, thread per (atom, lm)
__global__ void k_splines(int natoms, int nrad, int nlm, const double *__restrict__ sx, const double *__restrict__ U,
                          double *__restrict__ spl, float *__restrict__ spl32, double *__restrict__ work)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= natoms * nlm) return;
    const int n = nrad;
    const double *u = U + (size_t)id * n;      // u[i] at r_n[i] (decreasing r)
    double *Bc = work + (size_t)id * 3 * n, *Cc = Bc + n, *Yc = Cc + n;
#define YV(i) u[n - 1 - (i)]
    double h0 = sx[1] - sx[0], h1 = sx[2] - sx[1];
    double r0 = (YV(1) - YV(0)) / h0, r1 = (YV(2) - YV(1)) / h1;
    double B0 = h1 * (h0 + h1);
    Cc[0] = (h0 + h1) * (h0 + h1);
    Yc[0] = r0 * (3 * h0 * h1 + 2 * h1 * h1) + r1 * h0 * h0;
    Bc[0] = B0;
    // forward sweep fused with the system assembly (cspline.cpp:83-128)
    Cc[0] = Cc[0] / B0;
    Yc[0] = Yc[0] / B0;
    for (int i = 1; i < n - 1; ++i) {
        h0 = sx[i] - sx[i - 1];
        h1 = sx[i + 1] - sx[i];
        r0 = (YV(i) - YV(i - 1)) / h0;
        r1 = (YV(i + 1) - YV(i)) / h1;
        const double A = h1, B = 2 * (h0 + h1), C = h0, Yv = 3 * (r0 * h1 + r1 * h0);
        const double den = B - A * Cc[i - 1];
        Cc[i] = C / den;
        Yc[i] = (Yv - A * Yc[i - 1]) / den;
    }
    {
        const int i = n - 1;
        const double A = (h0 + h1) * (h0 + h1), B = h0 * (h0 + h1);
        const double Yv = r0 * h1 * h1 + r1 * (3 * h0 * h1 + 2 * h0 * h0);
        Yc[i] = (Yv - A * Yc[i - 1]) / (B - A * Cc[i - 1]);
    }
    // back substitution: derivatives D (stored in Bc)
    double *D = Bc;
    D[n - 1] = Yc[n - 1];
    for (int i = n - 1; i > 0; --i) D[i - 1] = Yc[i - 1] - Cc[i - 1] * D[i];
    const int a = id / nlm, lm = id % nlm;
    double *out = spl + (((size_t)a * nlm + lm) * n) * 4;
    float *out32 = spl32 + (((size_t)a * nlm + lm) * n) * 4;
    for (int i = 0; i < n - 1; ++i) {
        const double dx = 1.0 / (sx[i + 1] - sx[i]);
        const double dy = (YV(i + 1) - YV(i)) * dx;
        const double c0 = YV(i), c1 = D[i], c2 = dx * (3 * dy - 2 * D[i] - D[i + 1]),
                     c3 = dx * dx * (-2 * dy + D[i] + D[i + 1]);
        out[4 * i] = c0; out[4 * i + 1] = c1; out[4 * i + 2] = c2; out[4 * i + 3] = c3;
        out32[4 * i] = (float)c0; out32[4 * i + 1] = (float)c1; out32[4 * i + 2] = (float)c2; out32[4 * i + 3] = (float)c3;
    }
    // interval n-1: clamp value of the last knot
    out[4 * (n - 1)] = YV(n - 1); out[4 * (n - 1) + 1] = 0.0; out[4 * (n - 1) + 2] = 0.0; out[4 * (n - 1) + 3] = 0.0;
    out32[4 * (n - 1)] = (float)YV(n - 1); out32[4 * (n - 1) + 1] = 0.f; out32[4 * (n - 1) + 2] = 0.f; out32[4 * (n - 1) + 3] = 0.f;
#undef YV
}

template <typename T> __device__ __forceinline__ T tsqrt(T x);
template <> __device__ __forceinline__ double tsqrt<double>(double x) { return sqrt(x); }
template <> __device__ __forceinline__ float tsqrt<float>(float x) { return sqrtf(x); }
template <typename T> __device__ __forceinline__ T tacos(T x);
template <> __device__ __forceinline__ double tacos<double>(double x) { return acos(x); }
template <> __device__ __forceinline__ float tacos<float>(float x) { return acosf(x); }

// K5e: total potential on every point; writes V and cj = w V / 2
template <typename T>
__global__ void __launch_bounds__(128) k_vcross(size_t npts, size_t npad, int natoms, int nrad, int nang, int lmax,
                                                const double *__restrict__ atoms, const double *__restrict__ X,
                                                const double *__restrict__ Yc, const double *__restrict__ Zc,
                                                const double *__restrict__ W, const double *__restrict__ sx,
                                                const T *__restrict__ spl, const T *__restrict__ pre,
                                                const T *__restrict__ rec, const double *__restrict__ Vown,
                                                double *__restrict__ V, double *__restrict__ cj,
                                                float *__restrict__ cj32)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    if (p >= npts) { V[p] = 0.0; cj[p] = 0.0; cj32[p] = 0.f; return; }
    const int nlm = (lmax + 1) * (lmax + 1);
    const int N = nrad;
    const int a = (int)(p / ((size_t)nrad * nang));
    const double px = X[p], py = Yc[p], pz = Zc[p];
    const double sx0 = sx[0], sxN = sx[N - 1];
    const T fscale = T((double)(N + 1) / kPi);
    double Vt = 0.0;
    for (int k = 0; k < natoms; ++k) {
        if (k == a) { Vt += Vown[p]; continue; }
        const double dxd = px - atoms[4 * k], dyd = py - atoms[4 * k + 1], dzd = pz - atoms[4 * k + 2];
        const T dx = T(dxd), dy = T(dyd), dz = T(dzd);
        const T r = tsqrt<T>(dx * dx + dy * dy + dz * dz);
        const double rd = double(r);
        int iv;
        T t;
        if (rd < sx0) { iv = 0; t = T(0); }
        else if (rd >= sxN) { iv = N - 1; t = T(0); }
        else {
            // r <= sx[i] <=> radial index p(r) >= N - i, p(r) = acos((r-1)/(r+1)) (N+1)/pi
            const T pr = tacos<T>((r - T(1)) / (r + T(1))) * fscale;
            int i = (int)ceil(double(N) - double(pr));
            i = max(1, min(N - 1, i));
            while (i < N - 1 && rd > sx[i]) ++i;
            while (i > 1 && rd <= sx[i - 1]) --i;
            iv = i - 1;
            t = T(rd - sx[iv]);
        }
        const T inv_r = T(1) / r;
        const T ux = dx * inv_r, uy = dy * inv_r, uz = dz * inv_r;
        const T *cf = spl + ((size_t)k * nlm * N + iv) * 4;   // + lm*N*4
        T acc = T(0);
        T cm = T(1), sm = T(0);     // Re / Im of (ux + i uy)^m
        T qmm = T(1);               // Q_m^m = (-1)^m (2m-1)!!
        for (int m = 0; m <= lmax; ++m) {
            T q2 = T(0), q1 = qmm;
            for (int l = m; l <= lmax; ++l) {
                T q;
                if (l == m) q = qmm;
                else {
                    const int lmi = l * l + l + m;
                    q = rec[2 * lmi] * uz * q1 - rec[2 * lmi + 1] * q2;
                    q2 = q1;
                    q1 = q;
                }
                const int lp = l * l + l + m;
                const T *c0 = cf + (size_t)lp * N * 4;
                const T sp = c0[0] + t * (c0[1] + t * (c0[2] + t * c0[3]));
                if (m == 0) {
                    acc += pre[lp] * q * sp;
                } else {
                    const int ln = l * l + l - m;
                    const T *c1 = cf + (size_t)ln * N * 4;
                    const T sn = c1[0] + t * (c1[1] + t * (c1[2] + t * c1[3]));
                    acc += pre[lp] * q * cm * sp + pre[ln] * q * sm * sn;
                }
                if (l == m) { q2 = T(0); q1 = qmm; }
            }
            const T cn = cm * ux - sm * uy, sn2 = cm * uy + sm * ux;
            cm = cn; sm = sn2;
            qmm = -T(2 * m + 1) * qmm;
        }
        Vt += double(inv_r * acc);
    }
    V[p] = Vt;
    const double c = 0.5 * (W[p] * Vt);
    cj[p] = c;
    cj32[p] = (float)c;
}

int launch_hartree(dftg_ctx *c)
{
    const int N = c->nrad, S = N + 2, nlm = c->nlm;
    k_rholm<<<c->natoms * N, 128, sizeof(double) * c->nang, c->stream>>>(N, c->nang, nlm, c->d_rho, c->d_wb, c->d_Yw,
                                                                         c->d_rholm);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "rholm");
    const int nrhs = c->natoms * nlm;
    const size_t sm = sizeof(double) * S * 32;
    if (sm > 48 * 1024) DFTG_CUDA(cudaFuncSetAttribute(k_poisson, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    k_poisson<<<(nrhs + 31) / 32, 32, sm, c->stream>>>(c->natoms, N, c->lmax, c->d_rn, c->d_LU, c->d_piv, c->d_rholm,
                                                       c->d_scal, c->d_U);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "poisson");
    k_vown<<<(unsigned)((c->npts + 127) / 128), 128, 0, c->stream>>>(c->npts, N, c->nang, nlm, c->d_rn, c->d_leb,
                                                                     c->d_Y, c->d_U, c->d_Vown);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "vown");
    // the spline work area reuses the contraction partial buffer (3 * nrhs * N doubles)
    k_splines<<<(nrhs + 63) / 64, 64, 0, c->stream>>>(c->natoms, N, nlm, c->d_sx, c->d_U, c->d_spl, c->d_spl32,
                                                      c->d_part);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "splines");
    const unsigned nb = (unsigned)(c->npad / 128);
    if (c->precision == DFTG_PREC_FP64)
        k_vcross<double><<<nb, 128, 0, c->stream>>>(c->npts, c->npad, c->natoms, N, c->nang, c->lmax, c->d_atoms,
                                                    c->d_x, c->d_y, c->d_z, c->d_w, c->d_sx, c->d_spl, c->d_pre,
                                                    c->d_rec, c->d_Vown, c->d_V, c->d_cj, c->d_cj32);
    else
        k_vcross<float><<<nb, 128, 0, c->stream>>>(c->npts, c->npad, c->natoms, N, c->nang, c->lmax, c->d_atoms,
                                                   c->d_x, c->d_y, c->d_z, c->d_w, c->d_sx, c->d_spl32, c->d_pre32,
                                                   c->d_rec32, c->d_Vown, c->d_V, c->d_cj, c->d_cj32);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "vcross");
    return DFTG_OK;
}

}  // namespace dftg
