// k_integrals.cu -- K7: one-electron matrices S, T, V in FP64 on the device.
//
// Primitive integrals follow the reference's Obara-Saika / THO formulas:
// overlap through binomial prefactors (integrals.cpp:252-290), kinetic from
// shifted overlaps (integrals.cpp:101-121)
// and nuclear attraction through the A-array and the Boys function
// (integrals.cpp:336-387), with the truncated pi of integrals.cpp:342.
// Boys function F_m(x): the reference clamps x = max(|x|, 1e-8) and evaluates
// the incomplete gamma function with Numerical-Recipes routines (gamma.cpp);
// here F_mmax comes from the positive series e^-x sum (2x)^k / (2m+1)(2m+3)...
// (x < 40) followed by downward recursion, or from the erf closed form with
// upward recursion (x >= 40).
#include <cmath>
#include "dftg_internal.cuh"

namespace dftg {

__device__ __forceinline__ double fact_d(int n)
{
    double r = 1.0;
    for (int k = 2; k <= n; ++k) r *= k;
    return r;
}
__device__ __forceinline__ double dfact_d(int n)
{
    double r = 1.0;
    for (int k = n; k > 1; k -= 2) r *= k;
    return r;
}
__device__ __forceinline__ double ipow_i(double x, int n)
{
    double r = 1.0;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

__device__ double binomial_d(int a, int b)
{
    if ((a < 0) | (b < 0) | (a - b < 0)) return 1.0;
    return fact_d(a) / (fact_d(b) * fact_d(a - b));
}

__device__ double binomial_prefactor_d(int s, int ia, int ib, double xpa, double xpb)
{
    double sum = 0.0;
    for (int t = 0; t < s + 1; ++t)
        if ((s - ia <= t) && (t <= ib))
            sum += binomial_d(ia, s - t) * binomial_d(ib, t) * ipow_i(xpa, ia - s + t) * ipow_i(xpb, ib - t);
    return sum;
}

__device__ double overlap_1d_d(int l1, int l2, double x1, double x2, double gamma)
{
    double sum = 0.0;
    const int imax = 1 + (l1 + l2) / 2;
    for (int i = 0; i < imax; ++i)
        sum += binomial_prefactor_d(2 * i, l1, l2, x1, x2) * (i == 0 ? 1.0 : dfact_d(2 * i - 1)) / ipow_i(2 * gamma, i);
    return sum;
}

__device__ double ovl_prim_d(double a1, int l1, int m1, int n1, const double *A, double a2, int l2, int m2, int n2,
                             const double *B)
{
    const double g = a1 + a2;
    double rab2 = 0.0, P[3];
    for (int d = 0; d < 3; ++d) {
        rab2 += (A[d] - B[d]) * (A[d] - B[d]);
        P[d] = (a1 * A[d] + a2 * B[d]) / g;
    }
    const double pre = pow(kPi / g, 1.5) * exp(-a1 * a2 * rab2 / g);
    return pre * overlap_1d_d(l1, l2, P[0] - A[0], P[0] - B[0], g) * overlap_1d_d(m1, m2, P[1] - A[1], P[1] - B[1], g) *
           overlap_1d_d(n1, n2, P[2] - A[2], P[2] - B[2], g);
}

__device__ double kin_prim_d(double a1, int l1, int m1, int n1, const double *A, double a2, int l2, int m2, int n2,
                             const double *B)
{
    const double t0 = a2 * (2.0 * (l2 + m2 + n2) + 3.0) * ovl_prim_d(a1, l1, m1, n1, A, a2, l2, m2, n2, B);
    const double t1 = -2.0 * a2 * a2 *
                      (ovl_prim_d(a1, l1, m1, n1, A, a2, l2 + 2, m2, n2, B) + ovl_prim_d(a1, l1, m1, n1, A, a2, l2, m2 + 2, n2, B) +
                       ovl_prim_d(a1, l1, m1, n1, A, a2, l2, m2, n2 + 2, B));
    double t2 = 0.0;
    if (l2 >= 2) t2 += l2 * (l2 - 1) * ovl_prim_d(a1, l1, m1, n1, A, a2, l2 - 2, m2, n2, B);
    if (m2 >= 2) t2 += m2 * (m2 - 1) * ovl_prim_d(a1, l1, m1, n1, A, a2, l2, m2 - 2, n2, B);
    if (n2 >= 2) t2 += n2 * (n2 - 1) * ovl_prim_d(a1, l1, m1, n1, A, a2, l2, m2, n2 - 2, B);
    return t0 + t1 - 0.5 * t2;
}

// F_0..F_mmax at x (clamped as gamma.cpp:43)
__device__ void boys_all(int mmax, double x, double *F)
{
    x = fabs(x);
    if (x < 1e-8) x = 1e-8;
    const double ex = exp(-x);
    if (x < 40.0) {
        double term = 1.0 / (2 * mmax + 1), sum = term;
        for (int k = 1; k < 400; ++k) {
            term *= 2.0 * x / (2 * mmax + 2 * k + 1);
            sum += term;
            if (term < sum * 1e-17) break;
        }
        F[mmax] = ex * sum;
        for (int m = mmax - 1; m >= 0; --m) F[m] = (2.0 * x * F[m + 1] + ex) / (2 * m + 1);
    } else {
        F[0] = 0.5 * sqrt(kPi / x) * erf(sqrt(x));
        for (int m = 0; m < mmax; ++m) F[m + 1] = ((2 * m + 1) * F[m] - ex) / (2.0 * x);
    }
}

__device__ void a_array_d(int l1, int l2, double pa, double pb, double cp, double g, double *arr)
{
    const int imax = l1 + l2 + 1;
    for (int i = 0; i < imax; ++i) arr[i] = 0.0;
    for (int i = 0; i < imax; ++i)
        for (int r = 0; r <= i / 2; ++r)
            for (int u = 0; u <= (i - 2 * r) / 2; ++u) {
                const int iI = i - 2 * r - u;
                arr[iI] += ((i & 1) ? -1.0 : 1.0) * binomial_prefactor_d(i, l1, l2, pa, pb) * ((u & 1) ? -1.0 : 1.0) *
                           fact_d(i) * ipow_i(cp, i - 2 * r - 2 * u) * ipow_i(0.25 / g, r + u) / fact_d(r) / fact_d(u) /
                           fact_d(i - 2 * r - 2 * u);
            }
}

__device__ double nuc_prim_d(const double *A, int l1, int m1, int n1, double a1, const double *B, int l2, int m2, int n2,
                             double a2, const double *C)
{
    const double g = a1 + a2;
    double P[3], rab2 = 0.0, rcp2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        P[d] = (a1 * A[d] + a2 * B[d]) / g;
        rab2 += (A[d] - B[d]) * (A[d] - B[d]);
        rcp2 += (C[d] - P[d]) * (C[d] - P[d]);
    }
    double ax[9], ay[9], az[9], F[13];
    a_array_d(l1, l2, P[0] - A[0], P[0] - B[0], P[0] - C[0], g, ax);
    a_array_d(m1, m2, P[1] - A[1], P[1] - B[1], P[1] - C[1], g, ay);
    a_array_d(n1, n2, P[2] - A[2], P[2] - B[2], P[2] - C[2], g, az);
    const int mmax = l1 + l2 + m1 + m2 + n1 + n2;
    boys_all(mmax, rcp2 * g, F);
    double sum = 0.0;
    for (int i = 0; i <= l1 + l2; ++i)
        for (int j = 0; j <= m1 + m2; ++j)
            for (int k = 0; k <= n1 + n2; ++k) sum += ax[i] * ay[j] * az[k] * F[i + j + k];
    return -2.0 * kPiTrunc / g * exp(-a1 * a2 * rab2 / g) * sum;
}

// One warp per basis-function pair (i <= j); the lanes share the (primitive
// pair, nucleus) terms -- nucleus slot 0 carries the overlap and kinetic terms --
// and the warp sums them in a fixed shuffle order.
__global__ void __launch_bounds__(128) k_one_electron(int nbf, int natoms, const double *__restrict__ atoms,
                                                      const int *__restrict__ bf_lmn, const int *__restrict__ bf_off,
                                                      const int *__restrict__ bf_atom, const double *__restrict__ pa,
                                                      const double *__restrict__ pcn, double *S, double *T, double *V)
{
    const int id = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    const int npair = nbf * (nbf + 1) / 2;
    if (id >= npair) return;
    // id -> (i, j), i <= j, row-major over the upper triangle
    int i = 0, rem = id;
    while (rem >= nbf - i) { rem -= nbf - i; ++i; }
    const int j = i + rem;
    const int *qi = bf_lmn + 3 * i, *qj = bf_lmn + 3 * j;
    const double A[3] = {atoms[4 * bf_atom[i]], atoms[4 * bf_atom[i] + 1], atoms[4 * bf_atom[i] + 2]};
    const double B[3] = {atoms[4 * bf_atom[j]], atoms[4 * bf_atom[j] + 1], atoms[4 * bf_atom[j] + 2]};
    const int ki = bf_off[i], ni = bf_off[i + 1] - ki, kj = bf_off[j], nj = bf_off[j + 1] - kj;
    const int nterm = ni * nj * (natoms + 1);
    double s = 0.0, t = 0.0, v = 0.0;
    for (int e = lane; e < nterm; e += 32) {
        const int c = e / (ni * nj) - 1, pr = e % (ni * nj);
        const int k = ki + pr / nj, l = kj + pr % nj;
        const double pre = pcn[k] * pcn[l];
        if (c < 0) {
            s += pre * ovl_prim_d(pa[k], qi[0], qi[1], qi[2], A, pa[l], qj[0], qj[1], qj[2], B);
            t += pre * kin_prim_d(pa[k], qi[0], qi[1], qi[2], A, pa[l], qj[0], qj[1], qj[2], B);
        } else {
            const double C[3] = {atoms[4 * c], atoms[4 * c + 1], atoms[4 * c + 2]};
            v += atoms[4 * c + 3] * pre * nuc_prim_d(A, qi[0], qi[1], qi[2], pa[k], B, qj[0], qj[1], qj[2], pa[l], C);
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        s += __shfl_xor_sync(0xffffffffu, s, o);
        t += __shfl_xor_sync(0xffffffffu, t, o);
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    if (lane != 0) return;
    const size_t ij = (size_t)i + (size_t)j * nbf, ji = (size_t)j + (size_t)i * nbf;
    S[ij] = s; S[ji] = s;
    T[ij] = t; T[ji] = t;
    V[ij] = v; V[ji] = v;
}

int launch_one_electron(dftg_ctx *c, double *dS, double *dT, double *dV)
{
    const int npair = c->nbf * (c->nbf + 1) / 2;
    k_one_electron<<<(npair + 3) / 4, 128, 0, c->stream>>>(c->nbf, c->natoms, c->d_atoms, c->d_bf_lmn, c->d_bf_off,
                                                           c->d_bf_atom, c->d_pa, c->d_pcn, dS, dT, dV);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

}  // namespace dftg

extern "C" int dftg_one_electron(dftg_ctx *c, double *S, double *T, double *V)
{
    using namespace dftg;
    if (!c) { set_error("null context"); return DFTG_ERR_ARG; }
    if (c->points_only) { set_error("a point-set context has no nuclei"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    if (!c->d_ints_work) DFTG_CUDA(cudaMalloc(&c->d_ints_work, 3 * nn * sizeof(double)));
    double *dS = c->d_ints_work, *dT = dS + nn, *dV = dT + nn;
    int rc = launch_one_electron(c, dS, dT, dV);
    if (rc != DFTG_OK) return rc;
    if (S) DFTG_CUDA(cudaMemcpyAsync(S, dS, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (T) DFTG_CUDA(cudaMemcpyAsync(T, dT, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    if (V) DFTG_CUDA(cudaMemcpyAsync(V, dV, nn * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    return DFTG_OK;
}
