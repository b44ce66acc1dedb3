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
#include <algorithm>
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

// ------------------------------------------------------------------ two-electron integrals
//
// (ij|kl) over contracted Cartesian Gaussians for the reference's analytic
// Hartree path (DFT::calculate_two_electron_integrals dft.cpp:254-288,
// Integrator::repulsion integrals.cpp:185-466, which uses the
// Taketa-Huzinaga-O-ohata B-array).  Here the primitive integrals follow
// McMurchie and Davidson (J. Comput. Phys. 26 (1978) 218) in the form of
// Helgaker, Jorgensen and Olsen, "Molecular Electronic-Structure Theory" (2000)
// ch. 9: Hermite expansion coefficients E_t of each pair, the Hermite Coulomb
// integrals R_tuv by the downward recursion from (-2 alpha)^n F_n(alpha R_PQ^2),
// and (ab|cd) = 2 pi^(5/2) / (p q sqrt(p+q)) K_ab K_cd
//               sum_tuv E^ab_tuv sum_tau,nu,phi (-1)^(tau+nu+phi) E^cd R_(t+tau)(u+nu)(v+phi)
// with the truncated pi of integrals.cpp:394.  A formulation independent of the
// reference's, so agreement of the two is a check of both.  FP64 throughout.
namespace dftg {
namespace {

constexpr int kEriMaxL1 = 2;   // angular momentum per function (s, p, d)

// E^{la lb}_t, t = 0..la+lb, of one Cartesian direction (K_ab left out)
__device__ void herm_e(int la, int lb, double xpa, double xpb, double inv2p, double *e)
{
    double cur[2 * kEriMaxL1 + 2], nxt[2 * kEriMaxL1 + 2];
    for (int t = 0; t < 2 * kEriMaxL1 + 2; ++t) cur[t] = 0.0;
    cur[0] = 1.0;
    int n = 0;
    for (int s = 0; s < la + lb; ++s) {
        const double x = s < la ? xpa : xpb;
        for (int t = 0; t <= n + 1; ++t)
            nxt[t] = (t > 0 ? inv2p * cur[t - 1] : 0.0) + x * cur[t] + (t + 1 <= n ? (t + 1) * cur[t + 1] : 0.0);
        ++n;
        for (int t = 0; t <= n; ++t) cur[t] = nxt[t];
        cur[n + 1] = 0.0;
    }
    for (int t = 0; t <= la + lb; ++t) e[t] = cur[t];
}

template <int L>
__device__ __forceinline__ int ridx(int t, int u, int v) { return (t * (L + 1) + u) * (L + 1) + v; }

// contracted (ij|kl); L bounds the quartet's total angular momentum
template <int L>
__device__ double eri_contracted(int i, int j, int k, int l, const double *__restrict__ atoms,
                                 const int *__restrict__ bf_lmn, const int *__restrict__ bf_off,
                                 const int *__restrict__ bf_atom, const double *__restrict__ pa,
                                 const double *__restrict__ pcn)
{
    constexpr int N = (L + 1) * (L + 1) * (L + 1);
    const int fi[4] = {i, j, k, l};
    int lq[4][3];
    double ctr[4][3];
    for (int f = 0; f < 4; ++f)
        for (int d = 0; d < 3; ++d) {
            lq[f][d] = bf_lmn[3 * fi[f] + d];
            ctr[f][d] = atoms[4 * bf_atom[fi[f]] + d];
        }
    int ltot[3];
    for (int d = 0; d < 3; ++d) ltot[d] = lq[0][d] + lq[1][d] + lq[2][d] + lq[3][d];
    const int Lq = ltot[0] + ltot[1] + ltot[2];
    double rab2 = 0.0, rcd2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        rab2 += (ctr[0][d] - ctr[1][d]) * (ctr[0][d] - ctr[1][d]);
        rcd2 += (ctr[2][d] - ctr[3][d]) * (ctr[2][d] - ctr[3][d]);
    }
    const double two_pi52 = 2.0 * pow(kPiTrunc, 2.5);
    double sum = 0.0;
    double Ra[N], Rb[N], F[L + 1];
    double eab[3][2 * kEriMaxL1 + 1], ecd[3][2 * kEriMaxL1 + 1];
    for (int ka = bf_off[i]; ka < bf_off[i + 1]; ++ka)
        for (int kb = bf_off[j]; kb < bf_off[j + 1]; ++kb) {
            const double a = pa[ka], b = pa[kb], p = a + b;
            const double kab = exp(-a * b * rab2 / p);
            double Pc[3];
            for (int d = 0; d < 3; ++d) {
                Pc[d] = (a * ctr[0][d] + b * ctr[1][d]) / p;
                herm_e(lq[0][d], lq[1][d], Pc[d] - ctr[0][d], Pc[d] - ctr[1][d], 0.5 / p, eab[d]);
            }
            const double cab = pcn[ka] * pcn[kb] * kab;
            for (int kc = bf_off[k]; kc < bf_off[k + 1]; ++kc)
                for (int kd = bf_off[l]; kd < bf_off[l + 1]; ++kd) {
                    const double c = pa[kc], dd = pa[kd], q = c + dd;
                    const double kcd = exp(-c * dd * rcd2 / q);
                    double Qc[3], R[3];
                    for (int d = 0; d < 3; ++d) {
                        Qc[d] = (c * ctr[2][d] + dd * ctr[3][d]) / q;
                        herm_e(lq[2][d], lq[3][d], Qc[d] - ctr[2][d], Qc[d] - ctr[3][d], 0.5 / q, ecd[d]);
                        R[d] = Pc[d] - Qc[d];
                    }
                    const double alpha = p * q / (p + q);
                    const double rpq2 = R[0] * R[0] + R[1] * R[1] + R[2] * R[2];
                    boys_all(Lq, alpha * rpq2, F);
                    // R^n_tuv, n = Lq .. 0 (cur: level n + 1, nxt: level n)
                    double *cur = Ra, *nxt = Rb;
                    double m2a = 1.0;
                    for (int s = 0; s < Lq; ++s) m2a *= -2.0 * alpha;
                    cur[0] = m2a * F[Lq];
                    for (int n = Lq - 1; n >= 0; --n) {
                        m2a /= -2.0 * alpha;
                        nxt[0] = m2a * F[n];
                        const int top = Lq - n;
                        for (int t = 0; t <= top; ++t)
                            for (int u = 0; u <= top - t; ++u)
                                for (int v = 0; v <= top - t - u; ++v) {
                                    if (t + u + v == 0) continue;
                                    double r;
                                    if (t > 0)
                                        r = (t > 1 ? (t - 1) * cur[ridx<L>(t - 2, u, v)] : 0.0) +
                                            R[0] * cur[ridx<L>(t - 1, u, v)];
                                    else if (u > 0)
                                        r = (u > 1 ? (u - 1) * cur[ridx<L>(t, u - 2, v)] : 0.0) +
                                            R[1] * cur[ridx<L>(t, u - 1, v)];
                                    else
                                        r = (v > 1 ? (v - 1) * cur[ridx<L>(t, u, v - 2)] : 0.0) +
                                            R[2] * cur[ridx<L>(t, u, v - 1)];
                                    nxt[ridx<L>(t, u, v)] = r;
                                }
                        double *tmp = cur; cur = nxt; nxt = tmp;
                    }
                    // cur holds R^0_tuv
                    double acc = 0.0;
                    const int nab0 = lq[0][0] + lq[1][0], nab1 = lq[0][1] + lq[1][1], nab2 = lq[0][2] + lq[1][2];
                    const int ncd0 = lq[2][0] + lq[3][0], ncd1 = lq[2][1] + lq[3][1], ncd2 = lq[2][2] + lq[3][2];
                    for (int t = 0; t <= nab0; ++t)
                        for (int u = 0; u <= nab1; ++u)
                            for (int v = 0; v <= nab2; ++v) {
                                const double e1 = eab[0][t] * eab[1][u] * eab[2][v];
                                double inner = 0.0;
                                for (int tau = 0; tau <= ncd0; ++tau)
                                    for (int nu = 0; nu <= ncd1; ++nu)
                                        for (int ph = 0; ph <= ncd2; ++ph) {
                                            const double e2 = ecd[0][tau] * ecd[1][nu] * ecd[2][ph];
                                            const double sg = ((tau + nu + ph) & 1) ? -1.0 : 1.0;
                                            inner += sg * e2 * cur[ridx<L>(t + tau, u + nu, v + ph)];
                                        }
                                acc += e1 * inner;
                            }
                    sum += cab * pcn[kc] * pcn[kd] * kcd * two_pi52 / (p * q * sqrt(p + q)) * acc;
                }
        }
    return sum;
}

// pair index ij = i (i + 1) / 2 + j, i >= j (integrals.cpp:470-486)
__device__ __forceinline__ void pair_of(long long ij, int &i, int &j)
{
    long long r = (long long)((sqrt(8.0 * (double)ij + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > ij) --r;
    while ((r + 1) * (r + 2) / 2 <= ij) ++r;
    i = (int)r;
    j = (int)(ij - r * (r + 1) / 2);
}

// J_ij = sum_{k >= l} (2 - delta_kl) P_kl (ij|kl): block = 128 ket pairs of one bra pair
template <int L>
__global__ void __launch_bounds__(128) k_eri_j_partial(int nbf, int npair, const double *__restrict__ atoms,
                                                       const int *__restrict__ bf_lmn, const int *__restrict__ bf_off,
                                                       const int *__restrict__ bf_atom, const double *__restrict__ pa,
                                                       const double *__restrict__ pcn, const double *__restrict__ P,
                                                       double *__restrict__ part)
{
    __shared__ double sh[32];
    const int ij = blockIdx.y, kl = blockIdx.x * blockDim.x + threadIdx.x;
    double v = 0.0;
    if (kl < npair) {
        int i, j, k, l;
        pair_of(ij, i, j);
        pair_of(kl, k, l);
        const double w = (k == l ? 1.0 : 2.0) * P[k + (size_t)l * nbf];
        if (w != 0.0) v = w * eri_contracted<L>(i, j, k, l, atoms, bf_lmn, bf_off, bf_atom, pa, pcn);
    }
    v = block_sum(v, sh);
    if (threadIdx.x == 0) part[(size_t)ij * gridDim.x + blockIdx.x] = v;
}

__global__ void k_eri_j_reduce(int nbf, int npair, int nparts, const double *__restrict__ part, double *__restrict__ J)
{
    const int ij = blockIdx.x * blockDim.x + threadIdx.x;
    if (ij >= npair) return;
    double s = 0.0;
    for (int b = 0; b < nparts; ++b) s += part[(size_t)ij * nparts + b];
    int i, j;
    pair_of(ij, i, j);
    J[i + (size_t)j * nbf] = s;
    J[j + (size_t)i * nbf] = s;
}

// every unique (ij|kl), ij >= kl, at index ij (ij + 1) / 2 + kl
template <int L>
__global__ void __launch_bounds__(128) k_eri_list(int nbf, long long total, const double *__restrict__ atoms,
                                                  const int *__restrict__ bf_lmn, const int *__restrict__ bf_off,
                                                  const int *__restrict__ bf_atom, const double *__restrict__ pa,
                                                  const double *__restrict__ pcn, double *__restrict__ out)
{
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= total) return;
    int ij, kl, i, j, k, l;
    pair_of(id, ij, kl);
    pair_of(ij, i, j);
    pair_of(kl, k, l);
    out[id] = eri_contracted<L>(i, j, k, l, atoms, bf_lmn, bf_off, bf_atom, pa, pcn);
}

// total angular momentum bound of the basis: 4 (s, p) or 8 (d); -1 beyond d
int eri_lbound(const dftg_ctx *c)
{
    int lmax = 0;
    for (int f = 0; f < c->nbf; ++f) lmax = std::max(lmax, c->bf_lmn[3 * f] + c->bf_lmn[3 * f + 1] + c->bf_lmn[3 * f + 2]);
    if (lmax <= 1) return 4;
    if (lmax <= kEriMaxL1) return 8;
    return -1;
}

}  // namespace
}  // namespace dftg

extern "C" int dftg_eri_coulomb(dftg_ctx *c, const double *P, double *J)
{
    using namespace dftg;
    if (!c || !P || !J) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    if (c->points_only) { set_error("a point-set context has no molecular basis"); return DFTG_ERR_STATE; }
    const int L = eri_lbound(c);
    if (L < 0) { set_error("two-electron integrals support s, p and d functions"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    const int n = c->nbf, npair = n * (n + 1) / 2, nbx = (npair + 127) / 128;
    if (npair > 65535) { set_error("dftg_eri_coulomb supports nbf <= 361 (bra pairs on grid.y)"); return DFTG_ERR_ARG; }
    const size_t nn = (size_t)n * n;
    double *dP = nullptr, *dJ = nullptr, *dpart = nullptr;
    int rc = DFTG_OK;
    cudaError_t e = cudaMalloc(&dP, sizeof(double) * (2 * nn + (size_t)npair * nbx));
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    dJ = dP + nn;
    dpart = dJ + nn;
    e = cudaMemcpyAsync(dP, P, sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) {
        const dim3 grid(nbx, npair);
        if (L == 4)
            k_eri_j_partial<4><<<grid, 128, 0, c->stream>>>(n, npair, c->d_atoms, c->d_bf_lmn, c->d_bf_off,
                                                             c->d_bf_atom, c->d_pa, c->d_pcn, dP, dpart);
        else
            k_eri_j_partial<8><<<grid, 128, 0, c->stream>>>(n, npair, c->d_atoms, c->d_bf_lmn, c->d_bf_off,
                                                             c->d_bf_atom, c->d_pa, c->d_pcn, dP, dpart);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        k_eri_j_reduce<<<(npair + 127) / 128, 128, 0, c->stream>>>(n, npair, nbx, dpart, dJ);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(J, dJ, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = cuda_fail(e, "two-electron Coulomb matrix", __FILE__, __LINE__);
    cudaFree(dP);
    return rc;
}

extern "C" int dftg_eri_list(dftg_ctx *c, double *out, size_t cap)
{
    using namespace dftg;
    if (!c || !out) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    if (c->points_only) { set_error("a point-set context has no molecular basis"); return DFTG_ERR_STATE; }
    const int L = eri_lbound(c);
    if (L < 0) { set_error("two-electron integrals support s, p and d functions"); return DFTG_ERR_ARG; }
    const long long npair = (long long)c->nbf * (c->nbf + 1) / 2, total = npair * (npair + 1) / 2;
    if (cap < (size_t)total) { set_error("cap %zu < %lld integrals", cap, total); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    double *d = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(double) * total);
    if (e != cudaSuccess) return cuda_fail(e, "cudaMalloc", __FILE__, __LINE__);
    const unsigned nb = (unsigned)((total + 127) / 128);
    if (L == 4)
        k_eri_list<4><<<nb, 128, 0, c->stream>>>(c->nbf, total, c->d_atoms, c->d_bf_lmn, c->d_bf_off, c->d_bf_atom,
                                                 c->d_pa, c->d_pcn, d);
    else
        k_eri_list<8><<<nb, 128, 0, c->stream>>>(c->nbf, total, c->d_atoms, c->d_bf_lmn, c->d_bf_off, c->d_bf_atom,
                                                 c->d_pa, c->d_pcn, d);
    e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpyAsync(out, d, sizeof(double) * total, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    const int rc = e == cudaSuccess ? DFTG_OK : cuda_fail(e, "two-electron integral list", __FILE__, __LINE__);
    cudaFree(d);
    return rc;
}
