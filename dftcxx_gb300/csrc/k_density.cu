// k_density.cu -- density on the grid, charge reductions, LDA point kernel.
//
// K3  rho_p = 2 phi_p^T P phi_p (gridpoint.cpp:82-84).  One thread per point,
//     P staged in shared memory 32 columns at a time; T = double (FP64 path)
//     or float (mixed path, FP32 phi and P).  HBM traffic: nbf*npad*sizeof(T)
//     read once per 32-column block (the re-reads after the first hit L1/L2).
// K6  per-atom integrals q_a = sum_p w rho (atomicgrid.cpp:520-530), the
//     correction factor c = sum Z / sum q (moleculargrid.cpp:132-146) and the
//     rescaling rho <- c rho.  Deterministic two-stage FP64 reductions.
// LDA Slater exchange (functionals.cpp:24-63) + VWN correlation
//     (functionals.cpp:65-158), closed shell, fused with the weight: writes
//     cxc_p = w_p * v_p and block partials of E_xc = sum w (e_x + e_c).
#include "dftg_internal.cuh"
#include "lda_point.cuh"

namespace dftg {

constexpr int kRedBlock = 256;
constexpr int kRedChunk = 4096;   // points per stage-1 reduction block

template <typename T>
__global__ void __launch_bounds__(128) k_density(int nbf, size_t npad, const T *__restrict__ phi,
                                                 const T *__restrict__ P, double *__restrict__ rho)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T *Ps = reinterpret_cast<T *>(smem_raw);   // [nbf][32]
    const size_t p = (size_t)blockIdx.x * 128 + threadIdx.x;
    T r = 0;
    for (int n0 = 0; n0 < nbf; n0 += 32) {
        const int nc = min(32, nbf - n0);
        __syncthreads();
        for (int e = threadIdx.x; e < nbf * 32; e += 128) {
            const int mu = e >> 5, j = e & 31;
            Ps[e] = (j < nc) ? P[(size_t)mu * nbf + n0 + j] : T(0);
        }
        __syncthreads();
        T acc[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) acc[j] = 0;
        for (int mu = 0; mu < nbf; ++mu) {
            const T f = phi[(size_t)mu * npad + p];
            const T *pr = Ps + mu * 32;
#pragma unroll
            for (int j = 0; j < 32; ++j) acc[j] += f * pr[j];
        }
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (j < nc) r += acc[j] * phi[(size_t)(n0 + j) * npad + p];
    }
    rho[p] = 2.0 * (double)r;
}

// Mixed path of K3.  P enters as an FP32 hi/lo pair with separate accumulators
// (the FP32 rounding of P is common to every point and would bias the energy;
// the roundings of phi and of the accumulation differ point by point).  Each
// thread owns two points, so every P element read from shared memory feeds
// four FMAs.
__global__ void __launch_bounds__(128) k_density_split(int nbf, size_t npad, const float *__restrict__ phi,
                                                       const double *__restrict__ P, double *__restrict__ rho)
{
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *Ps = reinterpret_cast<float2 *>(smem_raw);   // [nbf][16] (hi, lo)
    const size_t p0 = (size_t)blockIdx.x * 256 + threadIdx.x, p1 = p0 + 128;
    const bool v1 = p1 < npad;
    float rh0 = 0.f, rl0 = 0.f, rh1 = 0.f, rl1 = 0.f;
    for (int n0 = 0; n0 < nbf; n0 += 16) {
        const int nc = min(16, nbf - n0);
        __syncthreads();
        for (int e = threadIdx.x; e < nbf * 16; e += 128) {
            const int mu = e >> 4, j = e & 15;
            float2 v = make_float2(0.f, 0.f);
            if (j < nc) {
                const double d = P[(size_t)mu * nbf + n0 + j];
                v.x = (float)d;
                v.y = (float)(d - (double)v.x);
            }
            Ps[e] = v;
        }
        __syncthreads();
        float ah0[16], al0[16], ah1[16], al1[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) { ah0[j] = 0.f; al0[j] = 0.f; ah1[j] = 0.f; al1[j] = 0.f; }
        for (int mu = 0; mu < nbf; ++mu) {
            const float f0 = phi[(size_t)mu * npad + p0];
            const float f1 = v1 ? phi[(size_t)mu * npad + p1] : 0.f;
            const float2 *pr = Ps + mu * 16;
#pragma unroll
            for (int j = 0; j < 16; ++j) {
                const float2 q = pr[j];
                ah0[j] = fmaf(f0, q.x, ah0[j]);
                al0[j] = fmaf(f0, q.y, al0[j]);
                ah1[j] = fmaf(f1, q.x, ah1[j]);
                al1[j] = fmaf(f1, q.y, al1[j]);
            }
        }
#pragma unroll
        for (int j = 0; j < 16; ++j)
            if (j < nc) {
                const float g0 = phi[(size_t)(n0 + j) * npad + p0];
                const float g1 = v1 ? phi[(size_t)(n0 + j) * npad + p1] : 0.f;
                rh0 = fmaf(ah0[j], g0, rh0);
                rl0 = fmaf(al0[j], g0, rl0);
                rh1 = fmaf(ah1[j], g1, rh1);
                rl1 = fmaf(al1[j], g1, rl1);
            }
    }
    rho[p0] = 2.0 * ((double)rh0 + (double)rl0);
    if (v1) rho[p1] = 2.0 * ((double)rh1 + (double)rl1);
}

// stage 1: partial sums of w*rho over chunks that never straddle two atoms
__global__ void __launch_bounds__(kRedBlock) k_atom_sums(size_t per_atom, int chunks_per_atom, int natoms,
                                                          const double *__restrict__ w, const double *__restrict__ rho,
                                                          double *__restrict__ part, const double *__restrict__ atoms,
                                                          double *scal, int mode, int *counter)
{
    __shared__ double sh[32];
    __shared__ double sq[kMaxAtoms];
    __shared__ int s_last;
    const int b = blockIdx.x;
    const int a = b / chunks_per_atom, ch = b % chunks_per_atom;
    const size_t base = (size_t)a * per_atom;
    const size_t lo = (size_t)ch * kRedChunk, hi = min(per_atom, lo + kRedChunk);
    double s = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += kRedBlock) s += w[base + i] * rho[base + i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[b] = s;
    if (!last_block(counter, &s_last)) return;
    // last block: per-atom sums in chunk order, total, correction factor
    for (int t = threadIdx.x; t < natoms; t += kRedBlock) {
        double q = 0.0;
        for (int c = 0; c < chunks_per_atom; ++c) q += __ldcg(part + (size_t)t * chunks_per_atom + c);
        sq[t] = q;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double total = 0.0, charge = 0.0;
        for (int t = 0; t < natoms; ++t) {
            total += sq[t];
            charge += atoms[4 * t + 3];
        }
        if (mode == 0) {           // before correction; charges scaled to the corrected density
            scal[kScalSum] = total;
            const double cf = charge / total;
            scal[kScalScale] = cf;
            double n = 0.0;
            for (int t = 0; t < natoms; ++t) {
                const double q = sq[t] * cf;
                scal[kScalAtomQ + t] = q;
                n += q;
            }
            scal[kScalNelec] = n;
        } else {                   // after correction
            for (int t = 0; t < natoms; ++t) scal[kScalAtomQ + t] = sq[t];
            scal[kScalNelec] = total;
        }
    }
}

__global__ void k_scale(size_t npts, const double *__restrict__ scal, double *rho)
{
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < npts) rho[p] *= scal[kScalScale];
}

// ---------------------------------------------------------------- LDA

template <bool MIXED>
__global__ void __launch_bounds__(kRedBlock) k_lda(size_t npad, double *__restrict__ rho,
                                                   const double *__restrict__ w, double *__restrict__ scal,
                                                   int apply_scale, double *__restrict__ cxc,
                                                   float *__restrict__ cxc32, double *__restrict__ part, int *counter,
                                                   int want64)
{
    __shared__ double sh[32];
    __shared__ float shf[2][32];
    __shared__ int s_last;
    const size_t p = (size_t)blockIdx.x * kRedBlock + threadIdx.x;
    double ew = 0.0;
    if (MIXED) {
        // double-float point kernel and block sum; FP64 only for the density
        // correction, the weight split and the block partial
        dfl ewd{0.f, 0.f};
        if (p < npad) {
            double r = rho[p];
            if (apply_scale) {
                r *= scal[kScalScale];
                rho[p] = r;
            }
            dfl e;
            float v;
            lda_point_df(df_from(r), e, v);
            const dfl wd = df_from(w[p]);
            ewd = df_mul(wd, e);
            const float c32 = (wd.h + wd.l) * v;
            cxc32[p] = c32;
            if (want64) cxc[p] = w[p] * (double)v;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
            ewd = df_add(ewd, dfl{__shfl_xor_sync(0xffffffffu, ewd.h, o), __shfl_xor_sync(0xffffffffu, ewd.l, o)});
        if ((threadIdx.x & 31) == 0) {
            shf[0][threadIdx.x >> 5] = ewd.h;
            shf[1][threadIdx.x >> 5] = ewd.l;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            dfl t{0.f, 0.f};
            for (int i = 0; i < kRedBlock / 32; ++i) t = df_add(t, dfl{shf[0][i], shf[1][i]});
            part[blockIdx.x] = df_to(t);
        }
        if (!last_block(counter, &s_last)) return;
        double t = 0.0;
        for (int i = threadIdx.x; i < (int)gridDim.x; i += kRedBlock) t += __ldcg(part + i);
        t = block_sum(t, sh);
        if (threadIdx.x == 0) scal[kScalExc] = t;
        return;
    }
    if (p < npad) {
        double r = rho[p];
        if (apply_scale) {        // density correction fused into the point kernel
            r *= scal[kScalScale];
            rho[p] = r;
        }
        double e;
        double vd;
        lda_point<double>(r, e, vd);
        const double wp = w[p];
        ew = wp * e;
        const double c = wp * vd;
        cxc[p] = c;
        cxc32[p] = (float)c;
    }
    ew = block_sum(ew, sh);
    if (threadIdx.x == 0) part[blockIdx.x] = ew;
    if (!last_block(counter, &s_last)) return;
    // last block: E_xc = sum of the block partials (fixed assignment and order)
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kRedBlock) t += __ldcg(part + i);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) scal[kScalExc] = t;
}

// ---------------------------------------------------------------- launchers

int launch_density(dftg_ctx *c)
{
    if (!(c->prec_mask & kPrecDensity)) {
        const unsigned nb = (unsigned)(c->npad / 128);
        const size_t sm = (size_t)c->nbf * 32 * sizeof(double);
        if (sm > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density<double>), c->device));
        k_density<double><<<nb, 128, sm, c->stream>>>(c->nbf, c->npad, c->d_phi, c->d_P, c->d_rho);
    } else if (c->tc_ready) {
        DFTG_TRY_L(launch_density_tc(c));
    } else {
        const unsigned nb = (unsigned)((c->npad + 255) / 256);
        const size_t sm = (size_t)c->nbf * 16 * sizeof(float2);
        if (sm > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density_split), c->device));
        k_density_split<<<nb, 128, sm, c->stream>>>(c->nbf, c->npad, c->d_phi32, c->d_P, c->d_rho);
    }
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "density");
    return DFTG_OK;
}

// kSumsOnly: per-atom charges of the current rho.  kSumsCorrect: correction
// factor, rho rescaled, charges recomputed (correct_densities).  kSumsFactor:
// correction factor and rescaled charges only; the LDA kernel rescales rho.
int launch_atom_sums(dftg_ctx *c, int mode)
{
    // a point-set context has one cell (all points) and no density correction
    if (c->points_only) mode = kSumsOnly;
    const int ncell = c->points_only ? 1 : c->natoms;
    const size_t per_atom = c->points_only ? c->npts : (size_t)c->nrad * c->nang;
    const int cpa = (int)((per_atom + kRedChunk - 1) / kRedChunk);
    const int nb = cpa * ncell;
    int *cnt = c->d_counters + kCntAtoms;
    k_atom_sums<<<nb, kRedBlock, 0, c->stream>>>(per_atom, cpa, ncell, c->d_w, c->d_rho, c->d_red, c->d_atoms,
                                                 c->d_scal, mode == kSumsOnly ? 1 : 0, cnt);
    DFTG_LAUNCH_CHECK();
    if (mode == kSumsCorrect) {
        k_scale<<<(unsigned)((c->npts + 255) / 256), 256, 0, c->stream>>>(c->npts, c->d_scal, c->d_rho);
        DFTG_LAUNCH_CHECK();
        k_atom_sums<<<nb, kRedBlock, 0, c->stream>>>(per_atom, cpa, c->natoms, c->d_w, c->d_rho, c->d_red, c->d_atoms,
                                                     c->d_scal, 1, cnt);
        DFTG_LAUNCH_CHECK();
    }
    DFTG_MARK(c, "charge");
    return DFTG_OK;
}

int launch_xc_points(dftg_ctx *c, bool apply_scale)
{
    const unsigned nb = (unsigned)((c->npad + kRedBlock - 1) / kRedBlock);
    const int sc = apply_scale ? 1 : 0;
    if (c->prec_mask & kPrecLda)
        k_lda<true><<<nb, kRedBlock, 0, c->stream>>>(c->npad, c->d_rho, c->d_w, c->d_scal, sc, c->d_cxc, c->d_cxc32,
                                                     c->d_red, c->d_counters + kCntLda,
                                                     (c->prec_mask & kPrecContract) && c->ct_ready ? 0 : 1);
    else
        k_lda<false><<<nb, kRedBlock, 0, c->stream>>>(c->npad, c->d_rho, c->d_w, c->d_scal, sc, c->d_cxc,
                                                      c->d_cxc32, c->d_red, c->d_counters + kCntLda, 1);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "lda");
    return DFTG_OK;
}

size_t reduction_elems(size_t npad, int natoms, int nrad, int nang)
{
    size_t a = (npad + kRedBlock - 1) / kRedBlock;
    size_t per_atom = (size_t)nrad * nang;
    size_t b = (size_t)natoms * ((per_atom + kRedChunk - 1) / kRedChunk);
    return a > b ? a : b;
}

}  // namespace dftg
