// k_adjoint.cu -- reverse-mode derivative (backward pass) of the grid energy
// of the last Fock build: dE/dP and dE/dR for
//   E = s_xc E_xc + s_j E_J,  E_xc = sum_p w_p e(rho_p),  E_J = 2 tr(P J) = sum_p (w_p V_p / 2) rho_raw,p
// exactly as the build evaluates them (dft.cpp:394-447, moleculargrid.cpp:132-146,
// 336-389, atomicgrid.cpp:241-556): rho_raw = 2 phi^T P phi, rho = c rho_raw with
// c = N / S, S = sum_p w_p rho_raw,p; V = A rho, A linear: projection on Y_lm
// (rho_lm = 4 pi sum_j rho w_becke w_leb Y_lm), the radial Poisson map with the
// l = 0 boundary charge q_a = sum_{p in a} w_p rho_p, the own-cell evaluation,
// the cubic-spline fit and the cross-atom evaluation.
//
// Backward (derived by hand, no tape):
//   u_p     = s_j w_p rho_raw,p
//   Abar    = A^T u: transposed cross-atom evaluation (pairs reduced per
//             (atom, spline interval) bin), transposed spline fit, transposed own-cell
//             evaluation, transposed Poisson map, transposed projection
//   g_p     = s_xc w_p v_p + Abar_p / 2,  gamma = sum_p g_p rho_p / S
//   h_p     = dE/drho_raw,p = s_j w_p V_p / 2 + c g_p - gamma w_p
//   dE/dP   = 2 phi^T diag(h) phi
//   dE/dR_C = sum_p h_p drho_raw,p/dR_C          (amplitudes: points move with their
//                                                 atom, functions with theirs)
//           + sum_p dE/dwb_p dwb_p/dR_C          (Becke weights)
//           + sum_(p,k) (u_p / 2) grad f_k(r_p - R_k) (delta_{C a(p)} - delta_{C k})
// with w_p = w0_p wb_p and
//   dE/dwb_p = w0_p (s_xc e_p + s_j rho_raw V / 2 + rho_p qbar_a / 2 - gamma rho_raw,p)
//              + rho_p mbar_p / 2.
// The FP64 kernels reduce per-atom force partials in a fixed order; the mixed
// kernels (FP32 per point or pair, FP64 or compensated FP32 sums) are listed
// below the FP64 ones.
#include <algorithm>
#include <cmath>
#include <vector>
#include "dftg_internal.cuh"
#include "lda_point.cuh"

namespace dftg {

constexpr int kBwBlock = 128;
constexpr int kBwRed = 256;

__global__ void k_bw_to_f32(int n, const double *__restrict__ a, const double *__restrict__ b, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[i] = (float)a[i];
        out[n + i] = (float)b[i];
    }
}

// pair (sorted place) -> grid point
__global__ void k_bw_pairpoint(size_t npts, int natoms, int per_atom, const int *__restrict__ pos,
                               int *__restrict__ pairp)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npts) return;
    const int a = (int)(p / per_atom);
    for (int k = 0; k < natoms; ++k)
        if (k != a) pairp[pos[p * natoms + k]] = (int)p;
}

// u = s_j w rho_raw (rho on the device carries the correction factor c)
__global__ void k_bw_seed(size_t npts, size_t npad, const double *__restrict__ rho, const double *__restrict__ w,
                          const double *__restrict__ scal, double sj, double *__restrict__ u)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    u[p] = p < npts ? sj * w[p] * (rho[p] / scal[kScalScale]) : 0.0;
}

// transposed own-cell evaluation: Ubar[a][lm][i] = sum_j u_p invr_p Y_lm(j)
__global__ void k_bw_own_T(int nrad, int nang, int nlm, const double *__restrict__ u, const double *__restrict__ invr,
                           const double *__restrict__ Y, double *__restrict__ Ubar)
{
    extern __shared__ double s_u[];   // [nang]
    const int a = blockIdx.x / nrad, i = blockIdx.x % nrad;
    const size_t base = ((size_t)a * nrad + i) * nang;
    for (int j = threadIdx.x; j < nang; j += blockDim.x) s_u[j] = u[base + j] * invr[base + j];
    __syncthreads();
    for (int lm = threadIdx.x; lm < nlm; lm += blockDim.x) {
        const double *y = Y + (size_t)lm * nang;
        double s = 0.0;
        for (int j = 0; j < nang; ++j) s += s_u[j] * y[j];
        Ubar[((size_t)a * nlm + lm) * nrad + i] = s;
    }
}

// Y_lm of a unit vector times the spherical-harmonic prefactor, in the order
// and recursion of the forward cross-atom evaluation: b[lm] for all lm.
__device__ __forceinline__ void bw_ylm(int lmax, double ux, double uy, double uz, const double *__restrict__ pre,
                                       const double *__restrict__ rec, double *b, int stride)
{
    double cm = 1.0, sm = 0.0, qmm = 1.0;
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
            if (m == 0) b[(size_t)lp * stride] = pre[lp] * q;
            else {
                const int ln = l * l + l - m;
                b[(size_t)lp * stride] = pre[lp] * q * cm;
                b[(size_t)ln * stride] = pre[ln] * q * sm;
            }
        }
        const double cn = cm * ux - sm * uy, sn = cm * uy + sm * ux;
        cm = cn;
        sm = sn;
        qmm = -(double)(2 * m + 1) * qmm;
    }
}

// Transposed cross-atom evaluation, one block per task (a run of at most 512
// pairs of one (atom k, spline interval) bin):
//   part[task][lm][n] = sum_pairs u_p / r Y_lm(dir) t^n,  n = 0..3
// 128 pairs at a time: their Y_lm go to shared memory, then thread lm sums.
__global__ void __launch_bounds__(kBwBlock) k_bw_cross_T(int nlm, int lmax, int nrad, const int4 *__restrict__ tasks,
                                                         const int *__restrict__ pairp, const double *__restrict__ atoms,
                                                         const double *__restrict__ X, const double *__restrict__ Yc,
                                                         const double *__restrict__ Zc, const double *__restrict__ u,
                                                         const double *__restrict__ sx, const double *__restrict__ pre,
                                                         const double *__restrict__ rec, double *__restrict__ part)
{
    constexpr int LDB = kBwBlock + 1;            // row stride: lanes reading different lm hit different banks
    extern __shared__ double s_b[];              // [nlm][LDB] then [4][128]
    double *s_t = s_b + (size_t)nlm * LDB;
    const int4 tk = tasks[blockIdx.x];
    const int k = tk.z, iv = tk.w, N = nrad;
    const double ax = atoms[4 * k], ay = atoms[4 * k + 1], az = atoms[4 * k + 2];
    double acc[2][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
    for (int q0 = 0; q0 < tk.y; q0 += kBwBlock) {
        const int q = q0 + threadIdx.x;
        if (q < tk.y) {
            const int p = pairp[tk.x + q];
            const double dx = X[p] - ax, dy = Yc[p] - ay, dz = Zc[p] - az;
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            const double inv_r = 1.0 / r;
            const double t = (r < sx[0] || r >= sx[N - 1]) ? 0.0 : r - sx[iv];
            const double s0 = u[p] * inv_r;
            s_t[threadIdx.x] = s0;
            s_t[kBwBlock + threadIdx.x] = s0 * t;
            s_t[2 * kBwBlock + threadIdx.x] = s0 * t * t;
            s_t[3 * kBwBlock + threadIdx.x] = s0 * t * t * t;
            bw_ylm(lmax, dx * inv_r, dy * inv_r, dz * inv_r, pre, rec, s_b + threadIdx.x, LDB);
        } else {
            for (int n = 0; n < 4; ++n) s_t[n * kBwBlock + threadIdx.x] = 0.0;
            for (int lm = 0; lm < nlm; ++lm) s_b[(size_t)lm * LDB + threadIdx.x] = 0.0;
        }
        __syncthreads();
        for (int s = 0; s < 2; ++s) {
            const int lm = threadIdx.x + s * kBwBlock;
            if (lm >= nlm) break;
            const double *b = s_b + (size_t)lm * LDB;
            double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
            for (int j = 0; j < kBwBlock; ++j) {
                const double bv = b[j];
                a0 += bv * s_t[j];
                a1 += bv * s_t[kBwBlock + j];
                a2 += bv * s_t[2 * kBwBlock + j];
                a3 += bv * s_t[3 * kBwBlock + j];
            }
            acc[s][0] += a0;
            acc[s][1] += a1;
            acc[s][2] += a2;
            acc[s][3] += a3;
        }
        __syncthreads();
    }
    for (int s = 0; s < 2; ++s) {
        const int lm = threadIdx.x + s * kBwBlock;
        if (lm >= nlm) break;
        double *o = part + ((size_t)blockIdx.x * nlm + lm) * 4;
        for (int n = 0; n < 4; ++n) o[n] = acc[s][n];
    }
}

// Transposed spline fit, one block per (atom, lm): sums the task partials of
// each interval bin (cbar[iv][n], the derivative of E by coefficient n of
// interval iv), maps them back through c = L(y, D), D = K y, and adds the
// result to Ubar (radial order of the grid: largest radius first).
__global__ void k_bw_spline_T(int nrad, int nlm, const int *__restrict__ bin_first, const double *__restrict__ part,
                              const double *__restrict__ splf, const double *__restrict__ Kt,
                              double *__restrict__ Ubar)
{
    extern __shared__ double s_c[];   // cbar [nrad][4], ybar [nrad], Dbar [nrad]
    const int id = blockIdx.x, k = id / nlm, lm = id % nlm, N = nrad;
    double *yb = s_c + 4 * N, *Db = yb + N;
    for (int iv = threadIdx.x; iv < N; iv += blockDim.x) {
        double c0 = 0.0, c1 = 0.0, c2 = 0.0, c3 = 0.0;
        const int t0 = bin_first[k * N + iv], t1 = bin_first[k * N + iv + 1];
        for (int t = t0; t < t1; ++t) {
            const double *q = part + ((size_t)t * nlm + lm) * 4;
            c0 += q[0];
            c1 += q[1];
            c2 += q[2];
            c3 += q[3];
        }
        s_c[4 * iv] = c0;
        s_c[4 * iv + 1] = c1;
        s_c[4 * iv + 2] = c2;
        s_c[4 * iv + 3] = c3;
    }
    __syncthreads();
    const double *inv_h = splf;
    // c0 = y_i, c1 = D_i, c2 = dx (3 dy - 2 D_i - D_{i+1}), c3 = dx^2 (-2 dy + D_i + D_{i+1}),
    // dy = (y_{i+1} - y_i) dx; the clamp interval N-1 holds c0 = y_{N-1}
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
        double y = 0.0, D = 0.0;
        if (i < N - 1) {
            const double dx = inv_h[i];
            const double dyb = 3.0 * dx * s_c[4 * i + 2] - 2.0 * dx * dx * s_c[4 * i + 3];
            y += s_c[4 * i] - dx * dyb;
            D += s_c[4 * i + 1] - 2.0 * dx * s_c[4 * i + 2] + dx * dx * s_c[4 * i + 3];
        } else {
            y += s_c[4 * i];
        }
        if (i > 0) {
            const int h = i - 1;
            const double dx = inv_h[h];
            const double dyb = 3.0 * dx * s_c[4 * h + 2] - 2.0 * dx * dx * s_c[4 * h + 3];
            y += dx * dyb;
            D += -dx * s_c[4 * h + 2] + dx * dx * s_c[4 * h + 3];
        }
        yb[i] = y;
        Db[i] = D;
    }
    __syncthreads();
    for (int j = threadIdx.x; j < N; j += blockDim.x) {
        double s = yb[j];
        const double *kr = Kt + (size_t)j * N;   // D_i = sum_j Kt[j][i] y_j
        for (int i = 0; i < N; ++i) s += kr[i] * Db[i];
        Ubar[(size_t)id * N + (N - 1 - j)] += s;
    }
}

// Transposed Poisson map, one block per (atom, lm):
//   rbar[k] = sum_i Gt[l][k][i] Ubar[i];  qbar_a = sum_i Gb[i] Ubar[a][0][i]
__global__ void k_bw_poisson_T(int nrad, int lmax, const double *__restrict__ Gt, const double *__restrict__ Gb,
                               const double *__restrict__ Ubar, double *__restrict__ rbar, double *__restrict__ qbar)
{
    extern __shared__ double s_ub[];   // [nrad]
    const int nlm = (lmax + 1) * (lmax + 1);
    const int id = blockIdx.x, a = id / nlm, lm = id % nlm, N = nrad;
    int l = 0;
    while ((l + 1) * (l + 1) <= lm) ++l;
    for (int i = threadIdx.x; i < N; i += blockDim.x) s_ub[i] = Ubar[(size_t)id * N + i];
    __syncthreads();
    const double *G = Gt + (size_t)l * N * N;
    for (int kk = threadIdx.x; kk < N; kk += blockDim.x) {
        const double *g = G + (size_t)kk * N;
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += g[i] * s_ub[i];
        rbar[(size_t)id * N + kk] = s;
    }
    if (lm == 0 && threadIdx.x == 0) {
        double s = 0.0;
        for (int i = 0; i < N; ++i) s += Gb[i] * s_ub[i];
        qbar[a] = s;
    }
}

// Per point: mbar (transposed projection), g = s_xc w v + (A^T u) / 2, the
// energy density e (with the point functions of the build's precision); block
// sums of g rho, the last block forms gamma.
template <bool MIXED>
__global__ void __launch_bounds__(kBwRed) k_bw_points(size_t npts, size_t npad, int nrad, int nang, int nlm,
                                                      const double *__restrict__ rho, const double *__restrict__ w,
                                                      const double *__restrict__ wb, const double *__restrict__ Yw,
                                                      const double *__restrict__ rbar, const double *__restrict__ qbar,
                                                      const double *__restrict__ scal, double sxc,
                                                      double *__restrict__ mbar, double *__restrict__ g,
                                                      double *__restrict__ e_out, double *__restrict__ red,
                                                      double *__restrict__ bw_scal, int *counter)
{
    __shared__ double sh[32];
    __shared__ int s_last;
    const size_t p = (size_t)blockIdx.x * kBwRed + threadIdx.x;
    double gr = 0.0;
    if (p < npad) {
        double mb = 0.0, gp = 0.0, ep = 0.0;
        if (p < npts) {
            const int per_atom = nrad * nang;
            const int a = (int)(p / per_atom), rem = (int)(p % per_atom), i = rem / nang, j = rem % nang;
            const double *rb = rbar + (size_t)a * nlm * nrad + i;
            for (int lm = 0; lm < nlm; ++lm) mb += Yw[(size_t)lm * nang + j] * rb[(size_t)lm * nrad];
            mb *= 4.0 * kPi;
            const double at = wb[p] * mb + w[p] * qbar[a];
            double v;
            if (MIXED) {   // the mixed point kernel of the build: FP32 potential, double-float energy
                dfl ed;
                float vf;
                lda_point_df(df_from(rho[p]), ed, vf);
                ep = df_to(ed);
                v = (double)vf;
            } else {
                lda_point<double>(rho[p], ep, v);
            }
            gp = sxc * w[p] * v + 0.5 * at;
            gr = gp * rho[p];
        }
        mbar[p] = mb;
        g[p] = gp;
        e_out[p] = ep;
    }
    gr = block_sum(gr, sh);
    if (threadIdx.x == 0) red[blockIdx.x] = gr;
    if (!last_block(counter, &s_last)) return;
    double t = 0.0;
    for (int b = threadIdx.x; b < (int)gridDim.x; b += kBwRed) t += __ldcg(red + b);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) bw_scal[0] = t / scal[kScalSum];
}

// Per point: h (the coefficient of drho_raw), 2 h (the contraction weight of
// dE/dP) and dE/dwb.
__global__ void k_bw_coef(size_t npts, size_t npad, int nrad, int nang, const double *__restrict__ rn,
                          const double *__restrict__ wrad, const double *__restrict__ leb,
                          const double *__restrict__ rho, const double *__restrict__ w, const double *__restrict__ V,
                          const double *__restrict__ g, const double *__restrict__ e, const double *__restrict__ mbar,
                          const double *__restrict__ qbar, const double *__restrict__ scal,
                          const double *__restrict__ bw_scal, double sxc, double sj, double *__restrict__ h,
                          double *__restrict__ h2, float *__restrict__ h2f, double *__restrict__ ewb)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    if (p >= npts) { h[p] = 0.0; h2[p] = 0.0; h2f[p] = 0.f; ewb[p] = 0.0; return; }
    const int per_atom = nrad * nang;
    const int a = (int)(p / per_atom), rem = (int)(p % per_atom), i = rem / nang, j = rem % nang;
    const double c = scal[kScalScale], gamma = bw_scal[0];
    const double r = rho[p], rr = r / c, wp = w[p], Vp = V[p];
    const double hp = sj * 0.5 * wp * Vp + c * g[p] - gamma * wp;
    h[p] = hp;
    h2[p] = 2.0 * hp;
    h2f[p] = (float)(2.0 * hp);
    // w0: the grid weight before the Becke factor, as the grid kernel forms it
    const double ri = rn[i];
    const double p2x = leb[4 * j] * ri, p2y = leb[4 * j + 1] * ri, p2z = leb[4 * j + 2] * ri;
    double w0 = wrad[i] * leb[4 * j + 3];
    w0 *= (p2x * p2x + p2y * p2y + p2z * p2z) * 4.0 * kPi;
    ewb[p] = w0 * (sxc * e[p] + sj * 0.5 * rr * Vp + 0.5 * r * qbar[a] - gamma * rr) + 0.5 * r * mbar[p];
}

// warp sum of a double (every lane gets it)
__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Adds each lane's vector v to acc[key] (key per lane; lanes with equal keys
// are summed first, in lane order).  acc: shared [..][3].
__device__ __forceinline__ void warp_add_by_key(int key, const double v[3], double *acc)
{
    const int lane = threadIdx.x & 31;
    unsigned todo = 0xffffffffu;
    while (todo) {
        const int leader = __ffs(todo) - 1;
        const int kl = __shfl_sync(0xffffffffu, key, leader);
        const unsigned grp = __ballot_sync(0xffffffffu, key == kl) & todo;
        double s[3];
        for (int c = 0; c < 3; ++c) s[c] = warp_sum_d((grp >> lane) & 1u ? v[c] : 0.0);
        if (lane == leader)
            for (int c = 0; c < 3; ++c) acc[3 * kl + c] += s[c];
        todo &= ~grp;
    }
}

// Amplitude term: sum_p h_p drho_raw,p/dR_C = sum_p 4 h_p sum_mu (P phi_p)_mu grad phi_mu
// (delta_{C a(p)} - delta_{C b(mu)}).  One thread per point, phi of the block
// in shared memory; per-warp per-atom accumulators.
__global__ void __launch_bounds__(kBwBlock) k_bw_force_phi(int nbf, int natoms, size_t npts, size_t npad, int per_atom,
                                                           const double *__restrict__ phi, const double *__restrict__ P,
                                                           const double *__restrict__ h, const double *__restrict__ X,
                                                           const double *__restrict__ Yc, const double *__restrict__ Zc,
                                                           const double *__restrict__ atoms,
                                                           const int *__restrict__ bf_lmn, const int *__restrict__ bf_off,
                                                           const int *__restrict__ bf_atom,
                                                           const double *__restrict__ pa, const double *__restrict__ pcn,
                                                           double *__restrict__ part)
{
    extern __shared__ double s_phi[];                       // [nbf][128], then [4][natoms][3]
    double *s_acc = s_phi + (size_t)nbf * kBwBlock;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t p = (size_t)blockIdx.x * kBwBlock + threadIdx.x;
    for (int nu = 0; nu < nbf; ++nu) s_phi[(size_t)nu * kBwBlock + threadIdx.x] = phi[(size_t)nu * npad + p];
    for (int e = threadIdx.x; e < 4 * natoms * 3; e += kBwBlock) s_acc[e] = 0.0;
    __syncthreads();
    const bool valid = p < npts;
    const int ap = valid ? (int)(p / per_atom) : 0;
    const double G = valid ? 4.0 * h[p] : 0.0;
    const double px = X[p], py = Yc[p], pz = Zc[p];
    double *acc = s_acc + (size_t)warp * natoms * 3;
    double self[3] = {0.0, 0.0, 0.0}, vb[3] = {0.0, 0.0, 0.0};
    int cur = bf_atom[0];
    auto flush = [&](int b) {
        double c[3];
        const bool use = valid && b != ap;
        for (int d = 0; d < 3; ++d) {
            c[d] = use ? G * vb[d] : 0.0;
            self[d] += c[d];
        }
        for (int d = 0; d < 3; ++d) {
            const double s = warp_sum_d(c[d]);
            if (lane == 0) acc[3 * b + d] -= s;
        }
    };
    for (int mu = 0; mu < nbf; ++mu) {
        const int b = bf_atom[mu];
        if (b != cur) {
            flush(cur);
            cur = b;
            vb[0] = vb[1] = vb[2] = 0.0;
        }
        const double *Pm = P + (size_t)mu * nbf;
        double t0 = 0.0, t1 = 0.0;
        int nu = 0;
        for (; nu + 1 < nbf; nu += 2) {
            t0 += Pm[nu] * s_phi[(size_t)nu * kBwBlock + threadIdx.x];
            t1 += Pm[nu + 1] * s_phi[(size_t)(nu + 1) * kBwBlock + threadIdx.x];
        }
        if (nu < nbf) t0 += Pm[nu] * s_phi[(size_t)nu * kBwBlock + threadIdx.x];
        const double t = t0 + t1;
        // gradient of the contracted Gaussian at p - R_b
        const double dx = px - atoms[4 * b], dy = py - atoms[4 * b + 1], dz = pz - atoms[4 * b + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const int lx = bf_lmn[3 * mu], ly = bf_lmn[3 * mu + 1], lz = bf_lmn[3 * mu + 2];
        double s0 = 0.0, s1 = 0.0;
        for (int k = bf_off[mu]; k < bf_off[mu + 1]; ++k) {
            const double ek = pcn[k] * exp(-pa[k] * r2);
            s0 += ek;
            s1 += pa[k] * ek;
        }
        double x0 = 1.0, y0 = 1.0, z0 = 1.0, xm = 0.0, ym = 0.0, zm = 0.0;
        for (int q = 0; q < lx; ++q) { xm = (q == lx - 1) ? (double)lx * x0 : xm; x0 *= dx; }
        for (int q = 0; q < ly; ++q) { ym = (q == ly - 1) ? (double)ly * y0 : ym; y0 *= dy; }
        for (int q = 0; q < lz; ++q) { zm = (q == lz - 1) ? (double)lz * z0 : zm; z0 *= dz; }
        const double gx = y0 * z0 * (xm * s0 - 2.0 * dx * x0 * s1);
        const double gy = x0 * z0 * (ym * s0 - 2.0 * dy * y0 * s1);
        const double gz = x0 * y0 * (zm * s0 - 2.0 * dz * z0 * s1);
        vb[0] += t * gx;
        vb[1] += t * gy;
        vb[2] += t * gz;
    }
    flush(cur);
    warp_add_by_key(ap, self, acc);
    __syncthreads();
    for (int e = threadIdx.x; e < natoms * 3; e += kBwBlock)
        part[(size_t)blockIdx.x * natoms * 3 + e] =
            ((s_acc[e] + s_acc[natoms * 3 + e]) + s_acc[2 * natoms * 3 + e]) + s_acc[3 * natoms * 3 + e];
}

// Becke smoothing step f(mu) = 3/2 mu - 1/2 mu^3 applied three times:
// s = (1 - f3) / 2 and ds/dmu (moleculargrid.cpp:310-329)
__device__ __forceinline__ void becke_s(double mu, double &s, double &ds)
{
    const double f1 = 1.5 * mu - 0.5 * (mu * mu * mu);
    const double f2 = 1.5 * f1 - 0.5 * (f1 * f1 * f1);
    const double f3 = 1.5 * f2 - 0.5 * (f2 * f2 * f2);
    s = 0.5 * (1.0 - f3);
    ds = -0.5 * (1.5 - 1.5 * f2 * f2) * (1.5 - 1.5 * f1 * f1) * (1.5 - 1.5 * mu * mu);
}

// same iteration as the grid kernel (for the cell functions themselves)
__device__ __forceinline__ double becke_s_fwd(double mu)
{
    for (int it = 0; it < 3; ++it) mu = 1.5 * mu - 0.5 * (mu * mu * mu);
    return 0.5 * (1.0 - mu);
}

// Becke-weight term: sum_p dE/dwb_p dwb_p/dR_C, wb = P_a / Z, P_B = prod_{k != B}
// s(mu_Bk), mu_Bk = (d_B - d_k) / R_Bk.  A warp per point, lanes over the cells
// B.  With the point held fixed, dmu_Bk/dR_B = (-e_B - mu e_Bk) / R_Bk and
// dmu_Bk/dR_k = (e_k + mu e_Bk) / R_Bk; the point moves with its atom a, which
// adds -sum over all atoms of those (translation invariance) to atom a.
__global__ void __launch_bounds__(kBwBlock) k_bw_force_becke(size_t npts, int per_atom, int natoms,
                                                             const double *__restrict__ atoms,
                                                             const double *__restrict__ rab,
                                                             const double *__restrict__ X, const double *__restrict__ Yc,
                                                             const double *__restrict__ Zc,
                                                             const double *__restrict__ ewb, double *__restrict__ part)
{
    extern __shared__ double s_m[];   // [4][natoms] d, [4][natoms] P, [4][natoms][3] acc
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *sd = s_m + (size_t)warp * natoms;
    double *sP = s_m + (size_t)(4 + warp) * natoms;
    double *s_accall = s_m + (size_t)8 * natoms;
    double *acc = s_accall + (size_t)warp * natoms * 3;
    for (int e = threadIdx.x; e < 4 * natoms * 3; e += kBwBlock) s_accall[e] = 0.0;
    __syncthreads();
    const size_t nw = (size_t)gridDim.x * 4;
    for (size_t p = (size_t)blockIdx.x * 4 + warp; p < npts; p += nw) {
        const double E = ewb[p];
        if (E == 0.0) continue;
        const int a = (int)(p / per_atom);
        const double px = X[p], py = Yc[p], pz = Zc[p];
        for (int k = lane; k < natoms; k += 32) {
            const double dx = px - atoms[4 * k], dy = py - atoms[4 * k + 1], dz = pz - atoms[4 * k + 2];
            sd[k] = sqrt(dx * dx + dy * dy + dz * dz);
        }
        __syncwarp();
        double zp = 0.0;
        for (int B = lane; B < natoms; B += 32) {
            double prod = 1.0;
            for (int k = 0; k < natoms; ++k) {
                if (k == B) continue;
                prod *= becke_s_fwd((sd[B] - sd[k]) / rab[B * natoms + k]);
            }
            sP[B] = prod;
            zp += prod;
        }
        const double Z = warp_sum_d(zp);
        __syncwarp();
        const double wb = sP[a] / Z;
        double tot[3] = {0.0, 0.0, 0.0};
        for (int B = lane; B < natoms; B += 32) {
            const double alpha = ((B == a ? 1.0 : 0.0) - wb) / Z;
            const double PB = sP[B];
            const double dB = sd[B];
            const double eBx = (px - atoms[4 * B]) / dB, eBy = (py - atoms[4 * B + 1]) / dB,
                         eBz = (pz - atoms[4 * B + 2]) / dB;
            double G[3] = {0.0, 0.0, 0.0};
            for (int tt = 1; tt < natoms; ++tt) {
                const int k = (B + tt) % natoms;
                const double Rbk = rab[B * natoms + k];
                const double mu = (dB - sd[k]) / Rbk;
                double s, ds;
                becke_s(mu, s, ds);
                double sigma;
                if (s > 1e-250) sigma = ds * (PB / s);
                else {
                    sigma = ds;
                    for (int k2 = 0; k2 < natoms; ++k2)
                        if (k2 != B && k2 != k) sigma *= becke_s_fwd((dB - sd[k2]) / rab[B * natoms + k2]);
                }
                const double coef = E * alpha * sigma / Rbk;
                if (coef == 0.0) continue;
                const double dk = sd[k];
                const double ekx = (px - atoms[4 * k]) / dk, eky = (py - atoms[4 * k + 1]) / dk,
                             ekz = (pz - atoms[4 * k + 2]) / dk;
                const double ebkx = (atoms[4 * B] - atoms[4 * k]) / Rbk, ebky = (atoms[4 * B + 1] - atoms[4 * k + 1]) / Rbk,
                             ebkz = (atoms[4 * B + 2] - atoms[4 * k + 2]) / Rbk;
                G[0] += coef * (-eBx - mu * ebkx);
                G[1] += coef * (-eBy - mu * ebky);
                G[2] += coef * (-eBz - mu * ebkz);
                atomicAdd(acc + 3 * k, coef * (ekx + mu * ebkx));
                atomicAdd(acc + 3 * k + 1, coef * (eky + mu * ebky));
                atomicAdd(acc + 3 * k + 2, coef * (ekz + mu * ebkz));
                tot[0] += coef * (ekx - eBx);
                tot[1] += coef * (eky - eBy);
                tot[2] += coef * (ekz - eBz);
            }
            atomicAdd(acc + 3 * B, G[0]);
            atomicAdd(acc + 3 * B + 1, G[1]);
            atomicAdd(acc + 3 * B + 2, G[2]);
        }
        for (int d = 0; d < 3; ++d) {
            const double s = warp_sum_d(tot[d]);
            if (lane == 0) acc[3 * a + d] -= s;
        }
        __syncwarp();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < natoms * 3; e += kBwBlock)
        part[(size_t)blockIdx.x * natoms * 3 + e] =
            ((s_accall[e] + s_accall[natoms * 3 + e]) + s_accall[2 * natoms * 3 + e]) + s_accall[3 * natoms * 3 + e];
}

// spline interval of r: smallest i >= 1 with r <= sx[i] (cspline.cpp:163-170),
// the rule of the forward evaluation (clamped ends give t = 0)
__device__ __forceinline__ void bw_interval(double rd, const double *__restrict__ sx, int N, double fscale, int &iv,
                                            double &t, bool &inside)
{
    inside = false;
    if (rd < sx[0]) { iv = 0; t = 0.0; return; }
    if (rd >= sx[N - 1]) { iv = N - 1; t = 0.0; return; }
    const float pr = acosf((float)((rd - 1.0) / (rd + 1.0))) * (float)fscale;
    int i = (int)ceilf((float)N - pr);
    i = max(1, min(N - 1, i));
    while (i < N - 1 && rd > sx[i]) ++i;
    while (i > 1 && rd <= sx[i - 1]) --i;
    iv = i - 1;
    t = rd - sx[iv];
    inside = true;
}

// Cross-atom geometry term: sum_(p, k != a) (u_p / 2) grad f_k(r_p - R_k), f_k(d) =
// (1/r) sum_lm S_klm(r) Y_lm(d / r); grad f = A1 u + (g - (u.g) u) / r^2 with
// A1 = sum (S'/r - S/r^2) Y, g = sum S grad_u Y (polynomial extension of Y in u).
__global__ void __launch_bounds__(kBwBlock) k_bw_force_cross(size_t npts, int natoms, int nrad, int per_atom, int lmax,
                                                             const double *__restrict__ atoms,
                                                             const double *__restrict__ X, const double *__restrict__ Yc,
                                                             const double *__restrict__ Zc, const double *__restrict__ u,
                                                             const double *__restrict__ sx,
                                                             const double *__restrict__ spl,
                                                             const double *__restrict__ pre,
                                                             const double *__restrict__ rec, double *__restrict__ part)
{
    extern __shared__ double s_a[];   // [4][natoms][3]
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *acc = s_a + (size_t)warp * natoms * 3;
    for (int e = threadIdx.x; e < 4 * natoms * 3; e += kBwBlock) s_a[e] = 0.0;
    __syncthreads();
    const size_t p = (size_t)blockIdx.x * kBwBlock + threadIdx.x;
    const bool valid = p < npts;
    const int ap = valid ? (int)(p / per_atom) : 0;
    const double coef = valid ? 0.5 * u[p] : 0.0;
    const double px = valid ? X[p] : 0.0, py = valid ? Yc[p] : 0.0, pz = valid ? Zc[p] : 0.0;
    const int nlm = (lmax + 1) * (lmax + 1), N = nrad;
    const double fscale = (double)(N + 1) / kPi;
    double self[3] = {0.0, 0.0, 0.0};
    for (int k = 0; k < natoms; ++k) {
        double vec[3] = {0.0, 0.0, 0.0};
        if (valid && k != ap && coef != 0.0) {
            const double dx = px - atoms[4 * k], dy = py - atoms[4 * k + 1], dz = pz - atoms[4 * k + 2];
            const double r = sqrt(dx * dx + dy * dy + dz * dz);
            int iv;
            double t;
            bool inside;
            bw_interval(r, sx, N, fscale, iv, t, inside);
            const double inv_r = 1.0 / r;
            const double ux = dx * inv_r, uy = dy * inv_r, uz = dz * inv_r;
            const double *cf = spl + ((size_t)k * nlm * N + iv) * 4;
            double A1 = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
            double cm = 1.0, sm = 0.0, cm1 = 0.0, sm1 = 0.0, qmm = 1.0;
            for (int m = 0; m <= lmax; ++m) {
                double q2 = 0.0, q1 = qmm, dq2 = 0.0, dq1 = 0.0;
                for (int l = m; l <= lmax; ++l) {
                    double q, dq;
                    if (l == m) { q = qmm; dq = 0.0; }
                    else {
                        const int lmi = l * l + l + m;
                        const double r0 = rec[2 * lmi], r1 = rec[2 * lmi + 1];
                        q = r0 * uz * q1 - r1 * q2;
                        dq = r0 * (q1 + uz * dq1) - r1 * dq2;
                        q2 = q1;
                        q1 = q;
                        dq2 = dq1;
                        dq1 = dq;
                    }
                    const int lp = l * l + l + m;
                    const double *c0 = cf + (size_t)lp * N * 4;
                    const double S = c0[0] + t * (c0[1] + t * (c0[2] + t * c0[3]));
                    const double Sp = inside ? c0[1] + t * (2.0 * c0[2] + 3.0 * t * c0[3]) : 0.0;
                    const double rad = Sp * inv_r - S * inv_r * inv_r;
                    if (m == 0) {
                        const double b = pre[lp] * q;
                        A1 += rad * b;
                        gz += S * pre[lp] * dq;
                    } else {
                        const double fm = (double)m;
                        const double bc = pre[lp] * q * cm;
                        A1 += rad * bc;
                        gx += S * pre[lp] * q * fm * cm1;
                        gy -= S * pre[lp] * q * fm * sm1;
                        gz += S * pre[lp] * dq * cm;
                        const int ln = l * l + l - m;
                        const double *c1 = cf + (size_t)ln * N * 4;
                        const double Sn = c1[0] + t * (c1[1] + t * (c1[2] + t * c1[3]));
                        const double Spn = inside ? c1[1] + t * (2.0 * c1[2] + 3.0 * t * c1[3]) : 0.0;
                        const double radn = Spn * inv_r - Sn * inv_r * inv_r;
                        A1 += radn * pre[ln] * q * sm;
                        gx += Sn * pre[ln] * q * fm * sm1;
                        gy += Sn * pre[ln] * q * fm * cm1;
                        gz += Sn * pre[ln] * dq * sm;
                    }
                }
                cm1 = cm;
                sm1 = sm;
                const double cn = cm * ux - sm * uy, sn = cm * uy + sm * ux;
                cm = cn;
                sm = sn;
                qmm = -(double)(2 * m + 1) * qmm;
            }
            const double ug = ux * gx + uy * gy + uz * gz;
            const double i2 = inv_r * inv_r;
            vec[0] = coef * (A1 * ux + i2 * (gx - ug * ux));
            vec[1] = coef * (A1 * uy + i2 * (gy - ug * uy));
            vec[2] = coef * (A1 * uz + i2 * (gz - ug * uz));
        }
        for (int d = 0; d < 3; ++d) {
            self[d] += vec[d];
            const double s = warp_sum_d(vec[d]);
            if (lane == 0) acc[3 * k + d] -= s;
        }
    }
    warp_add_by_key(ap, self, acc);
    __syncthreads();
    for (int e = threadIdx.x; e < natoms * 3; e += kBwBlock)
        part[(size_t)blockIdx.x * natoms * 3 + e] =
            ((s_a[e] + s_a[natoms * 3 + e]) + s_a[2 * natoms * 3 + e]) + s_a[3 * natoms * 3 + e];
}

// dEdR[a][c] = sum over the partial rows of the three force kernels: one block
// per element, fixed row assignment and order
__global__ void __launch_bounds__(256) k_bw_force_sum(int natoms, int nrows, const double *__restrict__ part,
                                                      double *__restrict__ dEdR)
{
    __shared__ double sh[32];
    const int e = blockIdx.x;
    double s = 0.0;
    for (int r = threadIdx.x; r < nrows; r += 256) s += part[(size_t)r * natoms * 3 + e];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) dEdR[e] = s;
}

// ---------------------------------------------------------------- mixed form
// FP32 arithmetic per point or pair, FP64 sums per block and across blocks.

// Becke cell function factors in factored form: with g_n = 1 - f_n and
// h_n = 1 + f_n, 1 - f(x) = (1 - x)^2 (2 + x) / 2 and 1 + f(x) = (1 + x)^2 (2 - x) / 2,
// so s(mu) = g_3 / 2 and s(-mu) = h_3 / 2 keep full relative precision down to
// underflow; ds/dmu = -(3/2)^3 (1 - mu^2) g_1 h_1 g_2 h_2 / 2 (the same for s(-mu)).
template <typename T>
__device__ __forceinline__ void becke_sT(T mu, T &s_p, T &s_m, T &ds)
{
    const T g0 = T(1) - mu, h0 = T(1) + mu;
    const T g1 = T(0.5) * g0 * g0 * (T(3) - g0), h1 = T(0.5) * h0 * h0 * (T(3) - h0);
    const T g2 = T(0.5) * g1 * g1 * (T(3) - g1), h2 = T(0.5) * h1 * h1 * (T(3) - h1);
    const T g3 = T(0.5) * g2 * g2 * (T(3) - g2), h3 = T(0.5) * h2 * h2 * (T(3) - h2);
    s_p = T(0.5) * g3;
    s_m = T(0.5) * h3;
    ds = T(-0.5 * 3.375) * (g0 * h0) * (g1 * h1) * (g2 * h2);
}

// Becke-weight term, a group of G lanes per point (32 / G points per warp),
// lane B of a group = cell B (natoms <= G).  Lane B forms P_B = prod_k s(mu_Bk)
// and, for every k != B (k = B + t mod n at step t, so the lanes' targets
// differ), coef = E alpha_B sigma_Bk / R_Bk: its own atom takes
// coef (-e_B - mu e_Bk) and atom k, through a shuffle, takes coef (e_k + mu e_Bk)
// (derivatives with the point held fixed).  Per point the lanes' vectors go to
// FP64 and the point's own atom takes minus their sum over the other atoms (the
// point moves with it), so each point adds exactly zero net force.
// T = float (mixed) or double.
template <typename T, int G>
__global__ void __launch_bounds__(kBwBlock) k_bw_becke_w(size_t npts, int per_atom, int natoms,
                                                         const double *__restrict__ atoms, const T *__restrict__ invR,
                                                         const T *__restrict__ ebk, const double *__restrict__ X,
                                                         const double *__restrict__ Yc, const double *__restrict__ Zc,
                                                         const double *__restrict__ ewb, double *__restrict__ part)
{
    constexpr int NG = 32 / G;
    __shared__ double s_acc[4][32][3];
    __shared__ T s_dist[4][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = lane / G, B0 = lane % G;
    const int n = natoms;
    const bool act = B0 < n;
    const int B = act ? B0 : 0;
    T *sd = s_dist[warp] + grp * G;
    const double ax = atoms[4 * B], ay = atoms[4 * B + 1], az = atoms[4 * B + 2];
    // per-lane totals: FP64 for T = double; a double-float (TwoSum) pair for
    // T = float, so no FP64 work runs per point
    double accx = 0.0, accy = 0.0, accz = 0.0;
    dfl fax{0.f, 0.f}, fay{0.f, 0.f}, faz{0.f, 0.f};
    const size_t stride = (size_t)gridDim.x * 4 * NG;
    for (size_t base = ((size_t)blockIdx.x * 4 + warp) * NG; base < npts; base += stride) {
        const size_t p = base + grp;
        const double Ed = p < npts ? ewb[p] : 0.0;
        const bool live = Ed != 0.0;
        const T E = (T)Ed;
        const int a = live ? (int)p / per_atom : 0;
        const T vx = live ? (T)(X[p] - ax) : T(1), vy = live ? (T)(Yc[p] - ay) : T(0),
                vz = live ? (T)(Zc[p] - az) : T(0);
        const T dB = act ? sqrt(vx * vx + vy * vy + vz * vz) : T(1);
        __syncwarp();
        sd[B0] = dB;
        __syncwarp();
        T PB = T(1);
        for (int k = 0; k < n; ++k)
            if (k != B) {
                T sp, sm, ds;
                becke_sT<T>((dB - sd[k]) * invR[B * n + k], sp, sm, ds);
                PB *= sp;
            }
        if (!act) PB = T(0);
        T Z = PB;
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) Z += __shfl_xor_sync(0xffffffffu, Z, o, G);
        const T iZ = T(1) / Z;
        const T wb = __shfl_sync(0xffffffffu, PB, a, G) * iZ;
        const T alB = ((B == a ? T(1) : T(0)) - wb) * iZ;
        const T iB = T(1) / dB;
        const T eBx = vx * iB, eBy = vy * iB, eBz = vz * iB;
        T Dx = T(0), Dy = T(0), Dz = T(0);
        int k = B, src = B;   // k = B + t, src = B - t (mod n)
        for (int t = 1; t < n; ++t) {
            k = k + 1 == n ? 0 : k + 1;
            src = src == 0 ? n - 1 : src - 1;
            const T ekx = __shfl_sync(0xffffffffu, eBx, k, G), eky = __shfl_sync(0xffffffffu, eBy, k, G),
                    ekz = __shfl_sync(0xffffffffu, eBz, k, G);
            T hx = T(0), hy = T(0), hz = T(0);
            if (act && live) {
                const T iR = invR[B * n + k];
                const T mu = (dB - sd[k]) * iR;
                T sp, sm, ds;
                becke_sT<T>(mu, sp, sm, ds);
                T sig;
                if (sp > (sizeof(T) == 4 ? T(1e-30) : T(1e-290))) sig = ds * (PB / sp);
                else {   // the factor underflows: product of the others
                    sig = ds;
                    for (int k2 = 0; k2 < n; ++k2)
                        if (k2 != B && k2 != k) {
                            T s2, m2, d2;
                            becke_sT<T>((dB - sd[k2]) * invR[B * n + k2], s2, m2, d2);
                            sig *= s2;
                        }
                }
                const T coef = E * alB * sig * iR;
                const T *u = ebk + 4 * ((size_t)B * n + k);
                Dx -= coef * (eBx + mu * u[0]);
                Dy -= coef * (eBy + mu * u[1]);
                Dz -= coef * (eBz + mu * u[2]);
                hx = coef * (ekx + mu * u[0]);
                hy = coef * (eky + mu * u[1]);
                hz = coef * (ekz + mu * u[2]);
            }
            Dx += __shfl_sync(0xffffffffu, hx, src, G);
            Dy += __shfl_sync(0xffffffffu, hy, src, G);
            Dz += __shfl_sync(0xffffffffu, hz, src, G);
        }
        // per point: other atoms take D, the owning atom minus their sum (exactly,
        // up to the final rounding: double-float sums for T = float)
        const bool other = act && live && B != a;
        if (sizeof(T) == 8) {
            double ox = other ? (double)Dx : 0.0, oy = other ? (double)Dy : 0.0, oz = other ? (double)Dz : 0.0;
            double sx = ox, sy = oy, sz = oz;
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) {
                sx += __shfl_xor_sync(0xffffffffu, sx, o, G);
                sy += __shfl_xor_sync(0xffffffffu, sy, o, G);
                sz += __shfl_xor_sync(0xffffffffu, sz, o, G);
            }
            if (other) { accx += ox; accy += oy; accz += oz; }
            else if (act && live) { accx -= sx; accy -= sy; accz -= sz; }
        } else {
            const float ox = other ? (float)Dx : 0.f, oy = other ? (float)Dy : 0.f, oz = other ? (float)Dz : 0.f;
            dfl sx{ox, 0.f}, sy{oy, 0.f}, sz{oz, 0.f};
#pragma unroll
            for (int o = G / 2; o > 0; o >>= 1) {
                sx = df_add(sx, dfl{__shfl_xor_sync(0xffffffffu, sx.h, o, G), __shfl_xor_sync(0xffffffffu, sx.l, o, G)});
                sy = df_add(sy, dfl{__shfl_xor_sync(0xffffffffu, sy.h, o, G), __shfl_xor_sync(0xffffffffu, sy.l, o, G)});
                sz = df_add(sz, dfl{__shfl_xor_sync(0xffffffffu, sz.h, o, G), __shfl_xor_sync(0xffffffffu, sz.l, o, G)});
            }
            if (other) {
                fax = df_add(fax, dfl{ox, 0.f});
                fay = df_add(fay, dfl{oy, 0.f});
                faz = df_add(faz, dfl{oz, 0.f});
            } else if (act && live) {
                fax = df_sub(fax, sx);
                fay = df_sub(fay, sy);
                faz = df_sub(faz, sz);
            }
        }
    }
    if (sizeof(T) == 4) {
        accx = df_to(fax);
        accy = df_to(fay);
        accz = df_to(faz);
    }
    s_acc[warp][lane][0] = accx;
    s_acc[warp][lane][1] = accy;
    s_acc[warp][lane][2] = accz;
    __syncthreads();
    for (int e = threadIdx.x; e < natoms * 3; e += kBwBlock) {
        const int at = e / 3, d = e % 3;
        double s = 0.0;
        for (int w = 0; w < 4; ++w)
            for (int g = 0; g < NG; ++g) s += s_acc[w][g * G + at][d];
        part[(size_t)blockIdx.x * natoms * 3 + e] = s;
    }
}

template <typename T>
static void launch_becke_w(dftg_ctx *c, int G, const T *iR, const T *eb, const double *ewb, double *fp)
{
    const int na = c->natoms, per_atom = c->nrad * c->nang;
    if (G == 8)
        k_bw_becke_w<T, 8><<<c->bw_nb_becke, kBwBlock, 0, c->stream>>>(c->npts, per_atom, na, c->d_atoms, iR, eb,
                                                                       c->d_x, c->d_y, c->d_z, ewb, fp);
    else if (G == 16)
        k_bw_becke_w<T, 16><<<c->bw_nb_becke, kBwBlock, 0, c->stream>>>(c->npts, per_atom, na, c->d_atoms, iR, eb,
                                                                        c->d_x, c->d_y, c->d_z, ewb, fp);
    else
        k_bw_becke_w<T, 32><<<c->bw_nb_becke, kBwBlock, 0, c->stream>>>(c->npts, per_atom, na, c->d_atoms, iR, eb,
                                                                        c->d_x, c->d_y, c->d_z, ewb, fp);
}

// Transposed cross-atom evaluation from the FP32 pair geometry and the integer
// Y_lm recursion of the mixed forward: part[task][lm][n] = fold_lm sum_pairs
// u_p / r R_lm(dir) t^n, FP32 sums over 128 pairs, FP64 across them.
__global__ void __launch_bounds__(kBwBlock) k_bw_cross_T32(int nlm, int lmax, const int4 *__restrict__ tasks,
                                                           const float4 *__restrict__ pgeo,
                                                           const float2 *__restrict__ ptk,
                                                           const int *__restrict__ pairp, const double *__restrict__ u,
                                                           const double *__restrict__ fold, double *__restrict__ part)
{
    constexpr int LDB = kBwBlock + 1;
    extern __shared__ float s_bf[];              // [nlm][LDB] then [4][128]
    float *s_t = s_bf + (size_t)nlm * LDB;
    const int4 tk = tasks[blockIdx.x];
    double acc[2][4] = {{0.0, 0.0, 0.0, 0.0}, {0.0, 0.0, 0.0, 0.0}};
    for (int q0 = 0; q0 < tk.y; q0 += kBwBlock) {
        const int q = q0 + threadIdx.x;
        float *b = s_bf + threadIdx.x;
        if (q < tk.y) {
            const float4 g = pgeo[(size_t)tk.x + q];
            const float t = ptk[(size_t)tk.x + q].x;
            const float s0 = (float)u[pairp[tk.x + q]] * g.w;
            s_t[threadIdx.x] = s0;
            s_t[kBwBlock + threadIdx.x] = s0 * t;
            s_t[2 * kBwBlock + threadIdx.x] = s0 * t * t;
            s_t[3 * kBwBlock + threadIdx.x] = s0 * t * t * t;
            float cm = 1.f, sm = 0.f;
            for (int m = 0; m <= lmax; ++m) {
                float r1 = 1.f, r2 = 0.f;
                for (int l = m; l <= lmax; ++l) {
                    float qv = 1.f;
                    if (l != m) {
                        qv = (float)(2 * l - 1) * g.z * r1 - (float)((l + m - 1) * (l - m - 1)) * r2;
                        r2 = r1;
                        r1 = qv;
                    }
                    if (m == 0) b[(size_t)(l * l + l) * LDB] = qv;
                    else {
                        b[(size_t)(l * l + l + m) * LDB] = qv * cm;
                        b[(size_t)(l * l + l - m) * LDB] = qv * sm;
                    }
                }
                const float cn = cm * g.x - sm * g.y, sn = cm * g.y + sm * g.x;
                cm = cn;
                sm = sn;
            }
        } else {
            for (int n = 0; n < 4; ++n) s_t[n * kBwBlock + threadIdx.x] = 0.f;
            for (int lm = 0; lm < nlm; ++lm) b[(size_t)lm * LDB] = 0.f;
        }
        __syncthreads();
        for (int s = 0; s < 2; ++s) {
            const int lm = threadIdx.x + s * kBwBlock;
            if (lm >= nlm) break;
            const float *bl = s_bf + (size_t)lm * LDB;
            float a0 = 0.f, a1 = 0.f, a2 = 0.f, a3 = 0.f;
#pragma unroll 4
            for (int j = 0; j < kBwBlock; ++j) {
                const float bv = bl[j];
                a0 = fmaf(bv, s_t[j], a0);
                a1 = fmaf(bv, s_t[kBwBlock + j], a1);
                a2 = fmaf(bv, s_t[2 * kBwBlock + j], a2);
                a3 = fmaf(bv, s_t[3 * kBwBlock + j], a3);
            }
            acc[s][0] += a0;
            acc[s][1] += a1;
            acc[s][2] += a2;
            acc[s][3] += a3;
        }
        __syncthreads();
    }
    for (int s = 0; s < 2; ++s) {
        const int lm = threadIdx.x + s * kBwBlock;
        if (lm >= nlm) break;
        double *o = part + ((size_t)blockIdx.x * nlm + lm) * 4;
        const double f = fold[lm];
        for (int n = 0; n < 4; ++n) o[n] = f * acc[s][n];
    }
}

// Cross-atom geometry term in FP32 over the pair bins (grid-stride over tasks):
// per pair (u_p / 2) grad f_k with the folded spline coefficients (high halves,
// plus the low halves for l = 0) and the integer Y_lm recursion; the bin's atom
// k takes minus the pair vectors, the pairs' own atoms take them: per pair slot
// the vectors are summed in FP32 over the lanes of each owning atom (runs of
// equal atom: the pairs of a bin are in point order) and that same sum goes, in
// FP64, to both atoms (exact translation sum rule, no FP64 work per pair).
__global__ void __launch_bounds__(kBwBlock) k_bw_force_cross32(int ntasks, int nlm, int lmax, int nrad, int natoms,
                                                               int per_atom, const int4 *__restrict__ tasks,
                                                               const float4 *__restrict__ pgeo,
                                                               const float2 *__restrict__ ptk,
                                                               const int *__restrict__ pairp,
                                                               const double *__restrict__ u,
                                                               const float *__restrict__ splm, double *__restrict__ part)
{
    extern __shared__ double s_x[];               // [4][natoms][3] doubles, then [nlm][2] float4 coefficients
    double *s_acc = s_x;
    float4 *s_cf = reinterpret_cast<float4 *>(s_x + 4 * (size_t)natoms * 3);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double *acc = s_acc + (size_t)warp * natoms * 3;
    for (int e = threadIdx.x; e < 4 * natoms * 3; e += kBwBlock) s_acc[e] = 0.0;
    for (int task = blockIdx.x; task < ntasks; task += gridDim.x) {
        const int4 tk = tasks[task];
        __syncthreads();
        for (int i = threadIdx.x; i < 2 * nlm; i += kBwBlock) {
            const int lm = i >> 1;
            s_cf[i] = reinterpret_cast<const float4 *>(splm + (((size_t)tk.z * nlm + lm) * nrad + tk.w) * 8)[i & 1];
        }
        __syncthreads();
        for (int q0 = 0; q0 < tk.y; q0 += kBwBlock) {
            const int q = q0 + threadIdx.x;
            float v[3] = {0.f, 0.f, 0.f};
            int key = -1;
            if (q < tk.y) {
                const float4 g = pgeo[(size_t)tk.x + q];
                const float t = ptk[(size_t)tk.x + q].x;
                const int p = pairp[tk.x + q];
                key = p / per_atom;
                const bool clamp = (tk.w == 0 && t == 0.f);   // below the first knot: constant
                const float ir = g.w, ir2 = ir * ir;
                float A1h = 0.f, A1l = 0.f, gx = 0.f, gy = 0.f, gz = 0.f;
                float cm = 1.f, sm = 0.f, cm1 = 0.f, sm1 = 0.f;
                for (int m = 0; m <= lmax; ++m) {
                    float r1 = 1.f, r2 = 0.f, d1 = 0.f, d2 = 0.f;
                    for (int l = m; l <= lmax; ++l) {
                        float qv = 1.f, dq = 0.f;
                        if (l != m) {
                            const float fa = (float)(2 * l - 1), fb = (float)((l + m - 1) * (l - m - 1));
                            qv = fa * g.z * r1 - fb * r2;
                            dq = fa * (r1 + g.z * d1) - fb * d2;
                            r2 = r1;
                            r1 = qv;
                            d2 = d1;
                            d1 = dq;
                        }
                        const float4 ch = s_cf[2 * (l * l + l + m)];
                        const float S = fmaf(t, fmaf(t, fmaf(t, ch.w, ch.z), ch.y), ch.x);
                        const float Sp = clamp ? 0.f : fmaf(t, fmaf(3.f * t, ch.w, 2.f * ch.z), ch.y);
                        if (m == 0) {
                            A1h = fmaf(qv, Sp * ir - S * ir2, A1h);
                            gz = fmaf(S, dq, gz);
                            if (l == 0) {
                                const float4 cl = s_cf[1];
                                const float Sl = fmaf(t, fmaf(t, fmaf(t, cl.w, cl.z), cl.y), cl.x);
                                const float Spl = clamp ? 0.f : fmaf(t, fmaf(3.f * t, cl.w, 2.f * cl.z), cl.y);
                                A1l = fmaf(qv, Spl * ir - Sl * ir2, A1l);
                            }
                        } else {
                            const float4 dh = s_cf[2 * (l * l + l - m)];
                            const float Sn = fmaf(t, fmaf(t, fmaf(t, dh.w, dh.z), dh.y), dh.x);
                            const float Spn = clamp ? 0.f : fmaf(t, fmaf(3.f * t, dh.w, 2.f * dh.z), dh.y);
                            const float fm = (float)m;
                            A1h = fmaf(qv * cm, Sp * ir - S * ir2, A1h);
                            A1h = fmaf(qv * sm, Spn * ir - Sn * ir2, A1h);
                            gx = fmaf(qv * fm, S * cm1 + Sn * sm1, gx);
                            gy = fmaf(qv * fm, Sn * cm1 - S * sm1, gy);
                            gz = fmaf(dq, S * cm + Sn * sm, gz);
                        }
                    }
                    cm1 = cm;
                    sm1 = sm;
                    const float cn = cm * g.x - sm * g.y, sn = cm * g.y + sm * g.x;
                    cm = cn;
                    sm = sn;
                }
                const float A1 = A1h + A1l;
                const float ug = g.x * gx + g.y * gy + g.z * gz;
                const float c = 0.5f * (float)u[p];
                v[0] = c * (A1 * g.x + ir2 * (gx - ug * g.x));
                v[1] = c * (A1 * g.y + ir2 * (gy - ug * g.y));
                v[2] = c * (A1 * g.z + ir2 * (gz - ug * g.z));
            }
            unsigned todo = 0xffffffffu;
            while (todo) {
                const int leader = __ffs(todo) - 1;
                const int kl = __shfl_sync(0xffffffffu, key, leader);
                const unsigned grp = __ballot_sync(0xffffffffu, key == kl) & todo;
                for (int d = 0; d < 3; ++d) {
                    float sv = (grp >> lane) & 1u ? v[d] : 0.f;
#pragma unroll
                    for (int o = 16; o > 0; o >>= 1) sv += __shfl_xor_sync(0xffffffffu, sv, o);
                    if (lane == leader && kl >= 0) {
                        acc[3 * kl + d] += (double)sv;
                        acc[3 * tk.z + d] -= (double)sv;
                    }
                }
                todo &= ~grp;
            }
        }
    }
    __syncthreads();
    for (int e = threadIdx.x; e < natoms * 3; e += kBwBlock)
        part[(size_t)blockIdx.x * natoms * 3 + e] =
            ((s_acc[e] + s_acc[natoms * 3 + e]) + s_acc[2 * natoms * 3 + e]) + s_acc[3 * natoms * 3 + e];
}

// Amplitude term in FP32 (one thread per point, FP32 phi and P in shared
// memory, (P phi)_mu formed four functions at a time from a broadcast row of
// P); per-atom vectors leave each point in FP64.
__global__ void __launch_bounds__(kBwBlock) k_bw_force_phi32(int nbf, int natoms, size_t npts, size_t npad,
                                                             int per_atom, const float *__restrict__ phi32,
                                                             const double *__restrict__ P, const double *__restrict__ h,
                                                             const double *__restrict__ X,
                                                             const double *__restrict__ Yc,
                                                             const double *__restrict__ Zc,
                                                             const double *__restrict__ atoms,
                                                             const int *__restrict__ bf_lmn,
                                                             const int *__restrict__ bf_off,
                                                             const int *__restrict__ bf_atom,
                                                             const float *__restrict__ pa,
                                                             const float *__restrict__ pcn, double *__restrict__ part)
{
    extern __shared__ double s_dd[];   // [4][natoms][3] doubles, [nbf][128] phi, [nbf][nbf4] P floats
    const int nbf4 = (nbf + 3) & ~3;
    double *s_acc = s_dd;
    float *s_phi = reinterpret_cast<float *>(s_dd + 4 * (size_t)natoms * 3);
    float *s_P = s_phi + (size_t)nbf * kBwBlock;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t p = (size_t)blockIdx.x * kBwBlock + threadIdx.x;
    for (int nu = 0; nu < nbf; ++nu) s_phi[(size_t)nu * kBwBlock + threadIdx.x] = phi32[(size_t)nu * npad + p];
    // s_P[nu][mu] = P(mu, nu) (P is symmetric; column-major element (mu, nu) at mu + nu nbf)
    for (int e = threadIdx.x; e < nbf * nbf4; e += kBwBlock) {
        const int nu = e / nbf4, mu = e % nbf4;
        s_P[e] = mu < nbf ? (float)P[(size_t)nu * nbf + mu] : 0.f;
    }
    for (int e = threadIdx.x; e < 4 * natoms * 3; e += kBwBlock) s_acc[e] = 0.0;
    __syncthreads();
    const bool valid = p < npts;
    const int ap = valid ? (int)(p / per_atom) : 0;
    const float G = valid ? (float)(4.0 * h[p]) : 0.f;
    const double px = X[p], py = Yc[p], pz = Zc[p];
    double *acc = s_acc + (size_t)warp * natoms * 3;
    float vb[3] = {0.f, 0.f, 0.f};
    int cur = bf_atom[0];
    float cx = 0.f, cy = 0.f, cz = 0.f;   // p - R_cur
    auto set_centre = [&](int b) {
        cx = (float)(px - atoms[4 * b]);
        cy = (float)(py - atoms[4 * b + 1]);
        cz = (float)(pz - atoms[4 * b + 2]);
    };
    // the point's vector for atom b (FP32, GB300's FP64 rate is low): summed in
    // FP32 over the warp's points of each owning atom (usually one), and that same
    // sum, once in FP64, taken from atom b and given to the owning atom, so the
    // term adds exactly zero net force
    auto flush = [&](int b) {
        const bool use = valid && b != ap;
        float c[3];
        for (int d = 0; d < 3; ++d) c[d] = use ? G * vb[d] : 0.f;
        unsigned todo = 0xffffffffu;
        while (todo) {
            const int leader = __ffs(todo) - 1;
            const int kl = __shfl_sync(0xffffffffu, ap, leader);
            const unsigned grp = __ballot_sync(0xffffffffu, ap == kl) & todo;
            for (int d = 0; d < 3; ++d) {
                float s = (grp >> lane) & 1u ? c[d] : 0.f;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
                if (lane == leader && kl != b) {
                    acc[3 * b + d] -= (double)s;
                    acc[3 * kl + d] += (double)s;
                }
            }
            todo &= ~grp;
        }
    };
    set_centre(cur);
    for (int mu0 = 0; mu0 < nbf; mu0 += 4) {
        float t[4] = {0.f, 0.f, 0.f, 0.f};
        for (int nu = 0; nu < nbf; ++nu) {
            const float f = s_phi[(size_t)nu * kBwBlock + threadIdx.x];
            const float4 pv = *reinterpret_cast<const float4 *>(s_P + (size_t)nu * nbf4 + mu0);
            t[0] = fmaf(pv.x, f, t[0]);
            t[1] = fmaf(pv.y, f, t[1]);
            t[2] = fmaf(pv.z, f, t[2]);
            t[3] = fmaf(pv.w, f, t[3]);
        }
        for (int j = 0; j < 4; ++j) {
            const int mu = mu0 + j;
            if (mu >= nbf) break;
            const int b = bf_atom[mu];
            if (b != cur) {
                flush(cur);
                cur = b;
                set_centre(b);
                vb[0] = vb[1] = vb[2] = 0.f;
            }
            const float r2 = cx * cx + cy * cy + cz * cz;
            const int lx = bf_lmn[3 * mu], ly = bf_lmn[3 * mu + 1], lz = bf_lmn[3 * mu + 2];
            float s0 = 0.f, s1 = 0.f;
            for (int k = bf_off[mu]; k < bf_off[mu + 1]; ++k) {
                const float al = pa[k];
                const float ek = pcn[k] * expf(-al * r2);
                s0 += ek;
                s1 = fmaf(al, ek, s1);
            }
            float x0 = 1.f, y0 = 1.f, z0 = 1.f, xm = 0.f, ym = 0.f, zm = 0.f;
            for (int q = 0; q < lx; ++q) { xm = (q == lx - 1) ? (float)lx * x0 : xm; x0 *= cx; }
            for (int q = 0; q < ly; ++q) { ym = (q == ly - 1) ? (float)ly * y0 : ym; y0 *= cy; }
            for (int q = 0; q < lz; ++q) { zm = (q == lz - 1) ? (float)lz * z0 : zm; z0 *= cz; }
            vb[0] = fmaf(t[j], y0 * z0 * (xm * s0 - 2.f * cx * x0 * s1), vb[0]);
            vb[1] = fmaf(t[j], x0 * z0 * (ym * s0 - 2.f * cy * y0 * s1), vb[1]);
            vb[2] = fmaf(t[j], x0 * y0 * (zm * s0 - 2.f * cz * z0 * s1), vb[2]);
        }
    }
    flush(cur);
    __syncthreads();
    for (int e = threadIdx.x; e < natoms * 3; e += kBwBlock)
        part[(size_t)blockIdx.x * natoms * 3 + e] =
            ((s_acc[e] + s_acc[natoms * 3 + e]) + s_acc[2 * natoms * 3 + e]) + s_acc[3 * natoms * 3 + e];
}

// ---------------------------------------------------------------- host side

static int bw_alloc(dftg_ctx *c)
{
    if (c->bw_ready) return DFTG_OK;
    const int N = c->nrad, nlm = c->nlm, na = c->natoms;
    const size_t rplane = (size_t)na * nlm * N;
    c->bw_nb_phi = (int)(c->npad / kBwBlock);
    c->bw_nb_becke = 152 * 8;
    c->bw_nb_cross = (int)(c->npad / kBwBlock);
    c->bw_nb_cross32 = std::max(1, std::min(c->ncross_tasks, 152 * 8));
    const size_t rows = (size_t)c->bw_nb_phi + c->bw_nb_becke + std::max(c->bw_nb_cross, c->bw_nb_cross32);
    const size_t nred = (c->npad + kBwRed - 1) / kBwRed;
    DFTG_CUDA(cudaMalloc(&c->d_bw_pt, sizeof(double) * 7 * c->npad + sizeof(float) * c->npad));
    {   // 1 / R_Bk, then the unit vectors (R_B - R_k) / R_Bk as [na * na][4], in FP32 and FP64
        const size_t nR = ((size_t)na * na + 3) / 4 * 4;
        std::vector<double> g64(nR + 4 * (size_t)na * na, 0.0);
        for (int B = 0; B < na; ++B)
            for (int k = 0; k < na; ++k) {
                if (B == k) continue;
                const double dx = c->xyz[3 * B] - c->xyz[3 * k], dy = c->xyz[3 * B + 1] - c->xyz[3 * k + 1],
                             dz = c->xyz[3 * B + 2] - c->xyz[3 * k + 2];
                const double R = std::sqrt(dx * dx + dy * dy + dz * dz);
                g64[(size_t)B * na + k] = 1.0 / R;
                double *e = g64.data() + nR + 4 * ((size_t)B * na + k);
                e[0] = dx / R;
                e[1] = dy / R;
                e[2] = dz / R;
            }
        std::vector<float> g32(g64.begin(), g64.end());
        DFTG_CUDA(cudaMalloc(&c->d_bw_geo, sizeof(float) * g32.size()));
        DFTG_CUDA(cudaMemcpy(c->d_bw_geo, g32.data(), sizeof(float) * g32.size(), cudaMemcpyHostToDevice));
        DFTG_CUDA(cudaMalloc(&c->d_bw_geo64, sizeof(double) * g64.size()));
        DFTG_CUDA(cudaMemcpy(c->d_bw_geo64, g64.data(), sizeof(double) * g64.size(), cudaMemcpyHostToDevice));
        c->bw_geo_off = (int)nR;
    }
    DFTG_CUDA(cudaMalloc(&c->d_bw_lm, sizeof(double) * (2 * rplane + na + 8 + nred)));
    DFTG_CUDA(cudaMalloc(&c->d_bw_fpart, sizeof(double) * rows * na * 3));
    if (!c->d_bw_out) DFTG_CUDA(cudaMalloc(&c->d_bw_out, sizeof(double) * ((size_t)c->nbf * c->nbf + (size_t)na * 3)));
    DFTG_CUDA(cudaMalloc(&c->d_bw_prim32, sizeof(float) * 2 * (size_t)std::max(1, c->nprim)));
    k_bw_to_f32<<<(unsigned)((c->nprim + 255) / 256 + 1), 256, 0, c->stream>>>(c->nprim, c->d_pa, c->d_pcn,
                                                                               c->d_bw_prim32);
    DFTG_LAUNCH_CHECK();
    DFTG_CUDA(cudaMalloc(&c->d_bw_counter, sizeof(int)));
    DFTG_CUDA(cudaMemsetAsync(c->d_bw_counter, 0, sizeof(int), c->stream));
    if (c->npairs > 0) {
        const int nt = c->ncross_tasks;
        DFTG_CUDA(cudaMalloc(&c->d_bw_pairp, sizeof(int) * c->npairs));
        DFTG_CUDA(cudaMalloc(&c->d_bw_binfirst, sizeof(int) * ((size_t)na * N + 1)));
        DFTG_CUDA(cudaMalloc(&c->d_bw_cpart, sizeof(double) * (size_t)nt * nlm * 4));
        k_bw_pairpoint<<<(unsigned)((c->npts + 255) / 256), 256, 0, c->stream>>>(c->npts, na, N * c->nang,
                                                                                 c->d_pairpos, c->d_bw_pairp);
        DFTG_LAUNCH_CHECK();
        std::vector<int4> tasks(nt);
        DFTG_CUDA(cudaMemcpyAsync(tasks.data(), c->d_cross_tasks, sizeof(int4) * nt, cudaMemcpyDeviceToHost,
                                  c->stream));
        DFTG_CUDA(cudaStreamSynchronize(c->stream));
        std::vector<int> first((size_t)na * N + 1, nt);
        for (int t = nt - 1; t >= 0; --t) first[(size_t)tasks[t].z * N + tasks[t].w] = t;
        for (int key = na * N - 1; key >= 0; --key)   // empty bins start where the next one does
            if (first[key] > first[key + 1]) first[key] = first[key + 1];
        DFTG_CUDA(cudaMemcpy(c->d_bw_binfirst, first.data(), sizeof(int) * first.size(), cudaMemcpyHostToDevice));
    }
    c->bw_ready = true;
    return DFTG_OK;
}

int launch_backward(dftg_ctx *c, double sxc, double sj, double *dEdP_dev, double *dEdR_dev)
{
    if (c->lmax > 13) {
        set_error("backward: lmax %d > 13", c->lmax);
        return DFTG_ERR_ARG;
    }
    DFTG_TRY_L(bw_alloc(c));
    const int N = c->nrad, nlm = c->nlm, na = c->natoms, nang = c->nang;
    const int per_atom = N * nang;
    const size_t rplane = (size_t)na * nlm * N;
    const size_t np = c->npad;
    double *u = c->d_bw_pt, *mbar = u + np, *g = mbar + np, *e = g + np, *h = e + np, *h2 = h + np, *ewb = h2 + np;
    double *Ubar = c->d_bw_lm, *rbar = Ubar + rplane, *qbar = rbar + rplane, *bws = qbar + na, *red = bws + 8;
    // the steps run in the precision of the build that produced the state: its
    // spline tables are current (FP64 ones whenever its cross-atom step was FP64)
    const unsigned mask = c->fwd_mask;
    const unsigned nb128 = (unsigned)(np / kBwBlock);
    const bool mx_cross = (mask & kPrecCross) != 0;
    const bool mx_phi = (mask & kPrecDensity) != 0;
    const bool mx_becke = (mask & kPrecLda) != 0;
    const bool mx_contract = (mask & kPrecContract) != 0;
    float *h2f = reinterpret_cast<float *>(c->d_bw_pt + 7 * np);
    const int4 *tasks = reinterpret_cast<const int4 *>(c->d_cross_tasks);
    const float4 *pgeo = reinterpret_cast<const float4 *>(c->d_pairs);
    const float2 *ptk = reinterpret_cast<const float2 *>(static_cast<const char *>(c->d_pairs) + sizeof(float4) * c->npairs);
    k_bw_seed<<<nb128, kBwBlock, 0, c->stream>>>(c->npts, np, c->d_rho, c->d_w, c->d_scal, sj, u);
    DFTG_LAUNCH_CHECK();
    k_bw_own_T<<<na * N, 96, sizeof(double) * nang, c->stream>>>(N, nang, nlm, u, c->d_invr, c->d_Y, Ubar);
    DFTG_LAUNCH_CHECK();
    if (c->npairs > 0) {
        if (mx_cross) {
            const size_t sm = sizeof(float) * ((size_t)nlm * (kBwBlock + 1) + 4 * kBwBlock);
            if (sm > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_cross_T32), c->device));
            k_bw_cross_T32<<<c->ncross_tasks, kBwBlock, sm, c->stream>>>(nlm, c->lmax, tasks, pgeo, ptk, c->d_bw_pairp,
                                                                          u, c->d_fold, c->d_bw_cpart);
        } else {
            const size_t sm = sizeof(double) * ((size_t)nlm * (kBwBlock + 1) + 4 * kBwBlock);
            if (sm > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_cross_T), c->device));
            k_bw_cross_T<<<c->ncross_tasks, kBwBlock, sm, c->stream>>>(nlm, c->lmax, N, tasks, c->d_bw_pairp,
                                                                        c->d_atoms, c->d_x, c->d_y, c->d_z, u, c->d_sx,
                                                                        c->d_pre, c->d_rec, c->d_bw_cpart);
        }
        DFTG_LAUNCH_CHECK();
        k_bw_spline_T<<<na * nlm, 128, sizeof(double) * 6 * N, c->stream>>>(N, nlm, c->d_bw_binfirst, c->d_bw_cpart,
                                                                            c->d_splf, c->d_Kt, Ubar);
        DFTG_LAUNCH_CHECK();
    }
    DFTG_MARK(c, "bw_cross_T");
    k_bw_poisson_T<<<na * nlm, 128, sizeof(double) * N, c->stream>>>(N, c->lmax, c->d_Gt, c->d_Gb, Ubar, rbar, qbar);
    DFTG_LAUNCH_CHECK();
    const unsigned nbr = (unsigned)((np + kBwRed - 1) / kBwRed);
    if (mask & kPrecLda)
        k_bw_points<true><<<nbr, kBwRed, 0, c->stream>>>(c->npts, np, N, nang, nlm, c->d_rho, c->d_w, c->d_wb, c->d_Yw,
                                                         rbar, qbar, c->d_scal, sxc, mbar, g, e, red, bws,
                                                         c->d_bw_counter);
    else
        k_bw_points<false><<<nbr, kBwRed, 0, c->stream>>>(c->npts, np, N, nang, nlm, c->d_rho, c->d_w, c->d_wb, c->d_Yw,
                                                          rbar, qbar, c->d_scal, sxc, mbar, g, e, red, bws,
                                                          c->d_bw_counter);
    DFTG_LAUNCH_CHECK();
    k_bw_coef<<<nb128, kBwBlock, 0, c->stream>>>(c->npts, np, N, nang, c->d_rn, c->d_wrad, c->d_leb, c->d_rho, c->d_w,
                                                 c->d_V, g, e, mbar, qbar, c->d_scal, bws, sxc, sj, h, h2, h2f, ewb);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "bw_points");
    if (dEdP_dev) {
        if (mx_contract && c->ct_ready) {
            DFTG_TRY_L(launch_contract_tc_on(c, h2f, h2f));
            DFTG_TRY_L(launch_contract_tc_reduce_to(c, true, false, dEdP_dev, nullptr));
        } else if (mx_contract) {
            DFTG_TRY_L(launch_contract_coef32(c, h2f, dEdP_dev));
        } else {
            DFTG_TRY_L(launch_contract_coef(c, h2, dEdP_dev));
        }
        DFTG_MARK(c, "bw_dEdP");
    }
    if (dEdR_dev) {
        double *fp = c->d_bw_fpart;
        int rows = 0;
        if (mx_phi) {
            const size_t smp = sizeof(double) * 4 * (size_t)na * 3 +
                               sizeof(float) * ((size_t)c->nbf * kBwBlock + (size_t)c->nbf * ((c->nbf + 3) & ~3));
            if (smp > 227 * 1024) {
                set_error("backward: nbf %d too large for the amplitude-gradient kernel", c->nbf);
                return DFTG_ERR_ARG;
            }
            if (smp > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_force_phi32), c->device));
            k_bw_force_phi32<<<c->bw_nb_phi, kBwBlock, smp, c->stream>>>(c->nbf, na, c->npts, np, per_atom, c->d_phi32,
                                                                         c->d_P, h, c->d_x, c->d_y, c->d_z, c->d_atoms,
                                                                         c->d_bf_lmn, c->d_bf_off, c->d_bf_atom,
                                                                         c->d_bw_prim32, c->d_bw_prim32 + c->nprim, fp);
        } else {
            const size_t smp = sizeof(double) * ((size_t)c->nbf * kBwBlock + 4 * (size_t)na * 3);
            if (smp > 227 * 1024) {
                set_error("backward: nbf %d too large for the amplitude-gradient kernel", c->nbf);
                return DFTG_ERR_ARG;
            }
            if (smp > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_force_phi), c->device));
            k_bw_force_phi<<<c->bw_nb_phi, kBwBlock, smp, c->stream>>>(c->nbf, na, c->npts, np, per_atom, c->d_phi,
                                                                       c->d_P, h, c->d_x, c->d_y, c->d_z, c->d_atoms,
                                                                       c->d_bf_lmn, c->d_bf_off, c->d_bf_atom, c->d_pa,
                                                                       c->d_pcn, fp);
        }
        DFTG_LAUNCH_CHECK();
        DFTG_MARK(c, "bw_force_phi");
        fp += (size_t)c->bw_nb_phi * na * 3;
        rows += c->bw_nb_phi;
        if (na <= 32) {
            const int G = na <= 8 ? 8 : (na <= 16 ? 16 : 32);
            if (mx_becke) {
                const float *iR = reinterpret_cast<const float *>(c->d_bw_geo);
                launch_becke_w<float>(c, G, iR, iR + c->bw_geo_off, ewb, fp);
            } else {
                const double *iR = c->d_bw_geo64;
                launch_becke_w<double>(c, G, iR, iR + c->bw_geo_off, ewb, fp);
            }
        } else {
            const size_t smb = sizeof(double) * 4 * (size_t)na * 5;
            if (smb > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_force_becke), c->device));
            k_bw_force_becke<<<c->bw_nb_becke, kBwBlock, smb, c->stream>>>(c->npts, per_atom, na, c->d_atoms, c->d_rab,
                                                                           c->d_x, c->d_y, c->d_z, ewb, fp);
        }
        DFTG_LAUNCH_CHECK();
        DFTG_MARK(c, "bw_force_becke");
        fp += (size_t)c->bw_nb_becke * na * 3;
        rows += c->bw_nb_becke;
        if (mx_cross) {
            if (c->npairs > 0) {
                const size_t smc = sizeof(double) * 4 * (size_t)na * 3 + sizeof(float4) * 2 * (size_t)nlm;
                if (smc > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_force_cross32), c->device));
                k_bw_force_cross32<<<c->bw_nb_cross32, kBwBlock, smc, c->stream>>>(
                    c->ncross_tasks, nlm, c->lmax, N, na, per_atom, tasks, pgeo, ptk, c->d_bw_pairp, u, c->d_splm, fp);
                DFTG_LAUNCH_CHECK();
                rows += c->bw_nb_cross32;
            }
        } else {
            const size_t smc = sizeof(double) * 4 * (size_t)na * 3;
            if (smc > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_bw_force_cross), c->device));
            k_bw_force_cross<<<c->bw_nb_cross, kBwBlock, smc, c->stream>>>(c->npts, na, N, per_atom, c->lmax, c->d_atoms,
                                                                           c->d_x, c->d_y, c->d_z, u, c->d_sx, c->d_spl,
                                                                           c->d_pre, c->d_rec, fp);
            DFTG_LAUNCH_CHECK();
            rows += c->bw_nb_cross;
        }
        DFTG_MARK(c, "bw_force_cross");
        k_bw_force_sum<<<(unsigned)(na * 3), 256, 0, c->stream>>>(na, rows, c->d_bw_fpart, dEdR_dev);
        DFTG_LAUNCH_CHECK();
    }
    return DFTG_OK;
}

}  // namespace dftg
