// k_grid.cu -- grid construction, Becke partition and basis amplitudes (FP64).
//
// K1: one thread per grid point: position, Gauss-Chebyshev x Lebedev weight
//     with the r^2 4pi Jacobian (atomicgrid.cpp:32-88) and the Becke fuzzy-cell
//     weight w_n = P_n / sum_m P_m, P_n = prod_{k!=n} s(mu_nk), s = (1 - f3)/2
//     (moleculargrid.cpp:229-254, 275-329).  FP64, O(natoms^2) per point.
// K2: one thread per (point, basis function): contracted Cartesian Gaussian
//     amplitude sum_k c_k N_k x^l y^m z^n exp(-alpha_k r^2) (cgf.cpp:49-57,
//     146-154), written as FP64 and FP32 planes [nbf][npad].
#include "dftg_internal.cuh"

namespace dftg {

__global__ void k_grid_points(int natoms, int cell0, const double *__restrict__ atoms, const double *__restrict__ rab,
                              int nrad, int nang, const double *__restrict__ rn, const double *__restrict__ wrad,
                              const double *__restrict__ leb, size_t npts, size_t npad,
                              double *X, double *Y, double *Zc, double *W, double *WB)
{
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    if (p >= npts) {   // padding: zero weight far away from everything
        X[p] = 0.0; Y[p] = 0.0; Zc[p] = 0.0; W[p] = 0.0; WB[p] = 0.0;
        return;
    }
    const int per_atom = nrad * nang;
    const int a = cell0 + (int)(p / per_atom);   // the cell (atom) that owns the point
    const int rem = (int)(p % per_atom);
    const int i = rem / nang;
    const int j = rem % nang;
    const double r = rn[i];
    const double p2x = leb[4 * j + 0] * r, p2y = leb[4 * j + 1] * r, p2z = leb[4 * j + 2] * r;
    const double px = atoms[4 * a + 0] + p2x, py = atoms[4 * a + 1] + p2y, pz = atoms[4 * a + 2] + p2z;
    double w = wrad[i] * leb[4 * j + 3];
    w *= (p2x * p2x + p2y * p2y + p2z * p2z) * 4.0 * kPi;

    // distances to every nucleus
    double d[kMaxAtoms];
    for (int k = 0; k < natoms; ++k) {
        double dx = px - atoms[4 * k], dy = py - atoms[4 * k + 1], dz = pz - atoms[4 * k + 2];
        d[k] = sqrt(dx * dx + dy * dy + dz * dz);
    }
    double denom = 0.0, nom = 1.0;
    for (int k = 0; k < natoms; ++k) {
        double wprod = 1.0;
        for (int m = 0; m < natoms; ++m) {
            if (m == k) continue;
            double mu = (d[k] - d[m]) / rab[k * natoms + m];
            for (int it = 0; it < 3; ++it) mu = 1.5 * mu - 0.5 * (mu * mu * mu);
            wprod *= 0.5 * (1.0 - mu);
        }
        denom += wprod;
        if (k == a) nom = wprod;
    }
    const double wb = nom / denom;
    X[p] = px; Y[p] = py; Zc[p] = pz;
    W[p] = w * wb;
    WB[p] = wb;
}

__device__ __forceinline__ double ipow_d(double x, int n)
{
    double r = 1.0;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

__global__ void k_amplitudes(int nbf, const int *__restrict__ bf_lmn, const int *__restrict__ bf_off,
                             const int *__restrict__ bf_atom, const double *__restrict__ atoms,
                             const double *__restrict__ pa, const double *__restrict__ pcn,
                             size_t npts, size_t npad, const double *__restrict__ X, const double *__restrict__ Y,
                             const double *__restrict__ Zc, double *phi, float *phi32)
{
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int mu = blockIdx.y;
    if (p >= npad) return;
    double v = 0.0;
    if (p < npts) {
        const int a = bf_atom[mu];
        const double dx = X[p] - atoms[4 * a], dy = Y[p] - atoms[4 * a + 1], dz = Zc[p] - atoms[4 * a + 2];
        const double r2 = dx * dx + dy * dy + dz * dz;
        const double ang = ipow_d(dx, bf_lmn[3 * mu]) * ipow_d(dy, bf_lmn[3 * mu + 1]) * ipow_d(dz, bf_lmn[3 * mu + 2]);
        for (int k = bf_off[mu]; k < bf_off[mu + 1]; ++k) v += pcn[k] * ang * exp(-pa[k] * r2);
    }
    phi[(size_t)mu * npad + p] = v;
    phi32[(size_t)mu * npad + p] = (float)v;
}

int launch_grid(dftg_ctx *c)
{
    const int bs = 128;
    const unsigned nb = (unsigned)((c->npad + bs - 1) / bs);
    k_grid_points<<<nb, bs, 0, c->stream>>>(c->natoms, c->cell0, c->d_atoms, c->d_rab, c->nrad, c->nang, c->d_rn, c->d_wrad,
                                            c->d_leb, c->npts, c->npad, c->d_x, c->d_y, c->d_z, c->d_w, c->d_wb);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int launch_amplitudes(dftg_ctx *c)
{
    const int bs = 256;
    dim3 grid((unsigned)((c->npad + bs - 1) / bs), (unsigned)c->nbf);
    k_amplitudes<<<grid, bs, 0, c->stream>>>(c->nbf, c->d_bf_lmn, c->d_bf_off, c->d_bf_atom, c->d_atoms, c->d_pa,
                                             c->d_pcn, c->npts, c->npad, c->d_x, c->d_y, c->d_z, c->d_phi,
                                             c->d_phi32);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

}  // namespace dftg
