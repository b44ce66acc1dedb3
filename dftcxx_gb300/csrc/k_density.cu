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
constexpr int kRedChunk = 1024;   // points per stage-1 reduction block (about two blocks per SM for benzene)

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

// P -> FP32 hi + lo (once per build; the density kernel stages from it), rows
// of ldp = nbf rounded up to 4 (16-byte rows), the padding zero
__global__ void k_split_P(int nbf, int ldp, const double *__restrict__ P, float *__restrict__ P32)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= nbf * ldp) return;
    const int mu = i / ldp, nu = i - mu * ldp;
    float h = 0.f, l = 0.f;
    if (nu < nbf) {
        const double d = P[(size_t)mu * nbf + nu];
        h = (float)d;
        l = (float)(d - (double)h);
    }
    P32[i] = h;
    P32[(size_t)nbf * ldp + i] = l;
}

// Mixed path of K3 on the CUDA cores (any nbf; the tensor-core form covers
// nbf <= 128).  P enters as an FP32 hi/lo pair with separate accumulators (the
// FP32 rounding of P is common to every point and would bias the energy; the
// roundings of phi and of the accumulation differ point by point).  Register
// tiling as in an SGEMM: a CTA takes 64 points and walks the columns of P in
// tiles of 128; a thread owns 4 points x 8 columns (hi and lo accumulators)
// fed from shared-memory stages of 32 basis functions (phi rows, P rows): 64
// FMAs per five 16-byte shared loads.  The stages are double-buffered with
// cp.async copies.  After a column tile each thread dots its eight columns with
// phi_nu at its points, the 16 column groups are summed in a fixed order and
// the tiles are summed in FP64.
constexpr int kDtPts = 64, kDtCols = 128, kDtK = 32, kDtThreads = 256;
struct DtStage {
    float phi[kDtK][kDtPts];
    float ph[kDtK][kDtCols];
    float pl[kDtK][kDtCols];
};
struct DtSmem {
    DtStage st[2];
    float red[2][kDtThreads / 16][kDtPts];
};

__device__ __forceinline__ void dt_cp16(float *dst, const float *src)
{
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}

// stage (column tile c0, basis functions k0..k0+31) into buffer s
__device__ __forceinline__ void dt_issue(DtStage &s, int nbf, int ldp, size_t npad, const float *phi,
                                         const float *P32, size_t p0, int c0, int k0, int tid)
{
    for (int e = tid; e < kDtK * kDtPts / 4; e += kDtThreads) {
        const int kk = e / (kDtPts / 4), q = e % (kDtPts / 4);
        float *d = &s.phi[kk][4 * q];
        if (k0 + kk < nbf) dt_cp16(d, phi + (size_t)(k0 + kk) * npad + p0 + 4 * q);
        else *reinterpret_cast<float4 *>(d) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    const size_t lo = (size_t)nbf * ldp;
    for (int e = tid; e < kDtK * kDtCols / 4; e += kDtThreads) {
        const int kk = e / (kDtCols / 4), q = e % (kDtCols / 4);
        const int mu = k0 + kk, nu = c0 + 4 * q;   // P symmetric: row mu read along nu
        float *dh = &s.ph[kk][4 * q], *dl = &s.pl[kk][4 * q];
        if (mu < nbf && nu < ldp) {
            const size_t o = (size_t)mu * ldp + nu;
            dt_cp16(dh, P32 + o);
            dt_cp16(dl, P32 + lo + o);
        } else {
            *reinterpret_cast<float4 *>(dh) = make_float4(0.f, 0.f, 0.f, 0.f);
            *reinterpret_cast<float4 *>(dl) = make_float4(0.f, 0.f, 0.f, 0.f);
        }
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__global__ void __launch_bounds__(kDtThreads) k_density_tiled(int nbf, int ldp, size_t npad,
                                                              const float *__restrict__ phi,
                                                              const float *__restrict__ P32, double *__restrict__ rho)
{
    extern __shared__ __align__(16) unsigned char dt_raw[];
    DtSmem &sm = *reinterpret_cast<DtSmem *>(dt_raw);
    const int tid = threadIdx.x, pg = tid & 15, cg = tid >> 4;   // points 4 pg .. +3, columns 8 cg .. +7
    const size_t p0 = (size_t)blockIdx.x * kDtPts;
    const int nk = (nbf + kDtK - 1) / kDtK, nc = (nbf + kDtCols - 1) / kDtCols, nstage = nk * nc;
    double rsum = 0.0;
    float ah[4][8], al[4][8];
    dt_issue(sm.st[0], nbf, ldp, npad, phi, P32, p0, 0, 0, tid);
    for (int s = 0; s < nstage; ++s) {
        const int ct = s / nk, kt = s - ct * nk;
        if (kt == 0) {
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) { ah[i][j] = 0.f; al[i][j] = 0.f; }
        }
        if (s + 1 < nstage) {
            const int ct1 = (s + 1) / nk, kt1 = s + 1 - ct1 * nk;
            dt_issue(sm.st[(s + 1) & 1], nbf, ldp, npad, phi, P32, p0, ct1 * kDtCols, kt1 * kDtK, tid);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        const DtStage &st = sm.st[s & 1];
#pragma unroll 4
        for (int kk = 0; kk < kDtK; ++kk) {
            const float4 f = *reinterpret_cast<const float4 *>(&st.phi[kk][4 * pg]);
            const float4 h0 = *reinterpret_cast<const float4 *>(&st.ph[kk][8 * cg]);
            const float4 h1 = *reinterpret_cast<const float4 *>(&st.ph[kk][8 * cg + 4]);
            const float4 l0 = *reinterpret_cast<const float4 *>(&st.pl[kk][8 * cg]);
            const float4 l1 = *reinterpret_cast<const float4 *>(&st.pl[kk][8 * cg + 4]);
            const float fv[4] = {f.x, f.y, f.z, f.w};
            const float hv[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
            const float lv[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) {
                    ah[i][j] = fmaf(fv[i], hv[j], ah[i][j]);
                    al[i][j] = fmaf(fv[i], lv[j], al[i][j]);
                }
        }
        __syncthreads();   // the buffer is refilled by the next prefetch
        if (kt == nk - 1) {
            // this column tile dotted with phi_nu at the thread's points
            const int c0 = ct * kDtCols;
            float sh[4] = {0.f, 0.f, 0.f, 0.f}, sl[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int nu = c0 + 8 * cg + j;
                if (nu < nbf) {
                    const float4 g = *reinterpret_cast<const float4 *>(phi + (size_t)nu * npad + p0 + 4 * pg);
                    const float gv[4] = {g.x, g.y, g.z, g.w};
#pragma unroll
                    for (int i = 0; i < 4; ++i) {
                        sh[i] = fmaf(ah[i][j], gv[i], sh[i]);
                        sl[i] = fmaf(al[i][j], gv[i], sl[i]);
                    }
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                sm.red[0][cg][4 * pg + i] = sh[i];
                sm.red[1][cg][4 * pg + i] = sl[i];
            }
            __syncthreads();
            if (tid < kDtPts) {
                float h = 0.f, l = 0.f;
                for (int g = 0; g < kDtThreads / 16; ++g) {
                    h += sm.red[0][g][tid];
                    l += sm.red[1][g][tid];
                }
                rsum += (double)h + (double)l;
            }
            __syncthreads();   // red is rewritten after the next column tile
        }
    }
    if (tid < kDtPts) rho[p0 + tid] = 2.0 * rsum;
}

// stage 1: partial sums of w*rho over chunks that never straddle two atoms;
// the last of the nb blocks sums them per atom and forms the correction factor
__device__ __forceinline__ void atom_sums_block(const SumsArgs A, int b, int nb)
{
    __shared__ double sh[32];
    __shared__ double sq[kMaxAtoms];
    __shared__ int s_last;
    const size_t per_atom = A.per_atom;
    const int chunks_per_atom = A.cpa, natoms = A.natoms;
    const double *__restrict__ w = A.w, *__restrict__ rho = A.rho;
    double *__restrict__ part = A.part;
    const int a = b / chunks_per_atom, ch = b % chunks_per_atom;
    const size_t base = (size_t)a * per_atom;
    const size_t lo = (size_t)ch * kRedChunk, hi = min(per_atom, lo + kRedChunk);
    double s = 0.0;
    for (size_t i = lo + threadIdx.x; i < hi; i += kRedBlock) s += w[base + i] * rho[base + i];
    s = block_sum(s, sh);
    if (threadIdx.x == 0) part[b] = s;
    if (!last_block_of(A.counter, nb, &s_last)) return;
    // last block: per-atom sums (a warp per atom: the lanes take every 32nd
    // chunk, then a fixed shuffle tree), total, correction factor
    {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        for (int t = warp; t < natoms; t += kRedBlock / 32) {
            double q = 0.0;
            for (int c = lane; c < chunks_per_atom; c += 32) q += __ldcg(part + (size_t)t * chunks_per_atom + c);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) q += __shfl_xor_sync(0xffffffffu, q, o);
            if (lane == 0) sq[t] = q;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double *scal = A.scal;
        double total = 0.0, charge = 0.0;
        for (int t = 0; t < natoms; ++t) {
            total += sq[t];
            charge += A.atoms[4 * t + 3];
        }
        if (A.mode == 0) {         // before correction; charges scaled to the corrected density
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
        if (A.done) {              // publish the factor to the grouped launch's point blocks
            __threadfence();
            flag_release(A.done, 1);
        }
    }
}

__global__ void __launch_bounds__(kRedBlock) k_atom_sums(const SumsArgs a)
{
    atom_sums_block(a, (int)blockIdx.x, (int)gridDim.x);
}

__global__ void k_scale(size_t npts, const double *__restrict__ scal, double *rho)
{
    size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < npts) rho[p] *= scal[kScalScale];
}

// ---------------------------------------------------------------- LDA

// Slater + VWN point kernel (functionals.cpp:24-114) with the density
// correction applied first when apply_scale (moleculargrid.cpp:132-146), E_xc
// summed per block and then over the blocks in order by the last one.  The
// mixed form with want_n also sums the integral of the corrected rho (the
// build's N, dft.cpp:111) and, with rw32, writes rho w_becke split into FP32
// hi / lo planes [2][npad] for the multipole kernel.
template <bool MIXED>
__device__ __forceinline__ void lda_block(const LdaArgs A, int vb, int nvb)
{
    const size_t npad = A.npad;
    double *__restrict__ rho = A.rho;
    const double *__restrict__ w = A.w;
    double *__restrict__ scal = A.scal;
    const int apply_scale = A.apply_scale, want64 = A.want64, want_n = A.want_n;
    double *__restrict__ cxc = A.cxc;
    float *__restrict__ cxc32 = A.cxc32;
    double *__restrict__ part = A.part;
    int *counter = A.counter;
    const double *__restrict__ wb = A.wb;
    float *__restrict__ rw32 = A.rw32;
    __shared__ double sh[32];
    __shared__ float shf[2][32], shn[2][32];
    __shared__ int s_last;
    const size_t p = (size_t)vb * kRedBlock + threadIdx.x;
    double ew = 0.0;
    if (MIXED) {
        // double-float point kernel and block sums; FP64 only for the density
        // correction (one product per point) and the block partials: rho is
        // split into FP32 hi / lo with integer operations, w and w_becke come as
        // FP32 hi / lo planes made at set-up
        dfl ewd{0.f, 0.f}, wrd{0.f, 0.f};
        float cbound = 0.f;                // |cxc32 / w| for the contraction's chunk bound
        if (p < npad) {
            double r = rho[p];
            if (apply_scale) {
                r *= __ldcg(scal + kScalScale);
                rho[p] = r;
            }
            const dfl rd = df_from_bits(r);
            dfl e;
            float v;
            lda_point_df(rd, e, v);
            const dfl wd{A.w2[p], A.w2[npad + p]};
            ewd = df_mul(wd, e);
            const float cv = (wd.h + wd.l) * v;
            cxc32[p] = cv;
            if (A.cmax) cbound = fabsf(cv) * A.winv[p];
            if (want64) cxc[p] = w[p] * (double)v;
            wrd = df_mul(wd, rd);
            if (rw32) {
                const dfl x = df_mul(rd, dfl{A.wb2[p], A.wb2[npad + p]});
                rw32[p] = x.h;
                rw32[npad + p] = x.l;
            }
        }
        if (A.cmax) warp_chunk_max(A.cmax, p < npad ? (int)(p / A.chunk_pts) : -1, cbound);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ewd = df_add(ewd, dfl{__shfl_xor_sync(0xffffffffu, ewd.h, o), __shfl_xor_sync(0xffffffffu, ewd.l, o)});
            wrd = df_add(wrd, dfl{__shfl_xor_sync(0xffffffffu, wrd.h, o), __shfl_xor_sync(0xffffffffu, wrd.l, o)});
        }
        if ((threadIdx.x & 31) == 0) {
            shf[0][threadIdx.x >> 5] = ewd.h;
            shf[1][threadIdx.x >> 5] = ewd.l;
            shn[0][threadIdx.x >> 5] = wrd.h;
            shn[1][threadIdx.x >> 5] = wrd.l;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            dfl t{0.f, 0.f}, tn{0.f, 0.f};
            for (int i = 0; i < kRedBlock / 32; ++i) {
                t = df_add(t, dfl{shf[0][i], shf[1][i]});
                tn = df_add(tn, dfl{shn[0][i], shn[1][i]});
            }
            part[vb] = df_to(t);
            if (want_n) part[nvb + vb] = df_to(tn);
        }
        if (!last_block_of(counter, nvb, &s_last)) return;
        double t = 0.0, tn = 0.0;
        for (int i = threadIdx.x; i < nvb; i += kRedBlock) {
            t += __ldcg(part + i);
            if (want_n) tn += __ldcg(part + nvb + i);
        }
        t = block_sum(t, sh);
        if (want_n) tn = block_sum(tn, sh);
        if (threadIdx.x == 0) {
            scal[kScalExc] = t;
            if (want_n) scal[kScalNelec] = tn;
        }
        return;
    }
    if (p < npad) {
        double r = rho[p];
        if (apply_scale) {        // density correction fused into the point kernel
            r *= __ldcg(scal + kScalScale);
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
    if (threadIdx.x == 0) part[vb] = ew;
    if (!last_block_of(counter, nvb, &s_last)) return;
    // last block: E_xc = sum of the block partials (fixed assignment and order)
    double t = 0.0;
    for (int i = threadIdx.x; i < nvb; i += kRedBlock) t += __ldcg(part + i);
    t = block_sum(t, sh);
    if (threadIdx.x == 0) scal[kScalExc] = t;
}

template <bool MIXED>
__global__ void __launch_bounds__(kRedBlock) k_lda(const LdaArgs a)
{
    pdl_wait();
    lda_block<MIXED>(a, (int)blockIdx.x, (int)gridDim.x);
    pdl_signal();
}

// The batch's per-atom sums and mixed point kernel in one persistent launch.
// Items [0, qs.nitems) are the molecules' atom-sum blocks, the next ql.nitems
// their point-kernel blocks, handed out from *head in that order.  A point block
// of molecule m first waits (bounded) until m's last atom-sum block has
// published the correction factor (done[m] = 1): every item it can wait on was
// handed out before it, to a running CTA, so the wait ends.  A wait that gives
// up records code 21 in *err and stops the CTA (the batch's results are then
// invalid).  A molecule without atom-sum items (its factor came from the
// P-slicing step) does not wait.  stall_mol >= 0 makes that molecule's point
// blocks wait for a value nothing writes (the self-test of the bounded wait).
__global__ void __launch_bounds__(kRedBlock) k_sums_lda_group(const SumsArgs *__restrict__ sa, GroupQueue qs,
                                                              const LdaArgs *__restrict__ la, GroupQueue ql,
                                                              SumsLdaCtl ctl)
{
    __shared__ int s_item, s_ok;
    const int total = qs.nitems + ql.nitems, take = ql.take;
    for (;;) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(ctl.head, take);
        __syncthreads();
        const int i0 = s_item;
        if (i0 >= total) return;
        const int i1 = min(total, i0 + take);
        for (int i = i0; i < i1; ++i) {
            if (i > i0) __syncthreads();
            if (i < qs.nitems) {
                const int m = gq_molecule(qs, i), b0 = __ldg(qs.prefix + m);
                const SumsArgs a = sa[m];
                atom_sums_block(a, i - b0, __ldg(qs.prefix + m + 1) - b0);
            } else {
                const int j = i - qs.nitems;
                const int m = gq_molecule(ql, j), b0 = __ldg(ql.prefix + m);
                // a molecule without atom-sum items has its factor already
                // (the P-slicing step); the self-test's molecule waits regardless
                const bool wait = m == ctl.stall_mol || __ldg(qs.prefix + m + 1) > __ldg(qs.prefix + m);
                if (wait && !wait_flag_ge(ctl.done + m, m == ctl.stall_mol ? 2 : 1, ctl.limit_ns, &s_ok)) {
                    if (threadIdx.x == 0) atomicExch(ctl.err, 21);
                    return;
                }
                const LdaArgs a = la[m];
                lda_block<true>(a, j - b0, __ldg(ql.prefix + m + 1) - b0);
            }
        }
    }
}

// ---------------------------------------------------------------- launchers

int launch_density(dftg_ctx *c, bool fused)
{
    c->rw_ready = false;             // a new density: the rho w_becke planes are stale
    if (!(c->prec_mask & kPrecDensity)) {
        const unsigned nb = (unsigned)(c->npad / 128);
        const size_t sm = (size_t)c->nbf * 32 * sizeof(double);
        if (sm > 48 * 1024) DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density<double>), c->device));
        k_density<double><<<nb, 128, sm, c->stream>>>(c->nbf, c->npad, c->d_phi, c->d_P, c->d_rho);
    } else if (c->tc_ready) {
        DFTG_TRY_L(launch_density_tc(c, fused));
    } else if (c->dt_ready) {
        DFTG_TRY_L(launch_density_tt(c));
    } else {
        const int ldp = (c->nbf + 3) / 4 * 4, n = c->nbf * ldp;
        k_split_P<<<(n + 255) / 256, 256, 0, c->stream>>>(c->nbf, ldp, c->d_P, c->d_P32);
        DFTG_LAUNCH_CHECK();
        DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density_tiled), c->device));
        k_density_tiled<<<(unsigned)(c->npad / kDtPts), kDtThreads, sizeof(DtSmem), c->stream>>>(
            c->nbf, ldp, c->npad, c->d_phi32, c->d_P32, c->d_rho);
    }
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "density");
    return DFTG_OK;
}

StepLaunch<SumsArgs> step_atom_sums(const dftg_ctx *c, int mode)
{
    // a point-set context has one cell (all points) and no density correction
    const int ncell = c->points_only ? 1 : c->ncell;
    const size_t per_atom = c->points_only ? c->npts : (size_t)c->nrad * c->nang;
    const int cpa = (int)((per_atom + kRedChunk - 1) / kRedChunk);
    StepLaunch<SumsArgs> s;
    s.args = SumsArgs{per_atom, cpa, ncell, mode == kSumsOnly || c->points_only ? 1 : 0, c->d_w, c->d_rho, c->d_red,
                      c->d_atoms, c->d_scal, c->d_counters + kCntAtoms, nullptr};
    s.blocks = cpa * ncell;
    return s;
}

// kSumsOnly: per-atom charges of the current rho.  kSumsCorrect: correction
// factor, rho rescaled, charges recomputed (correct_densities).  kSumsFactor:
// correction factor and rescaled charges only; the LDA kernel rescales rho.
int launch_atom_sums(dftg_ctx *c, int mode)
{
    if (c->points_only) mode = kSumsOnly;
    StepLaunch<SumsArgs> st = step_atom_sums(c, mode);
    k_atom_sums<<<st.blocks, kRedBlock, 0, c->stream>>>(st.args);
    DFTG_LAUNCH_CHECK();
    if (mode == kSumsCorrect) {
        c->rw_ready = false;         // rho is rescaled below
        k_scale<<<(unsigned)((c->npts + 255) / 256), 256, 0, c->stream>>>(c->npts, c->d_scal, c->d_rho);
        DFTG_LAUNCH_CHECK();
        st.args.mode = 1;
        k_atom_sums<<<st.blocks, kRedBlock, 0, c->stream>>>(st.args);
        DFTG_LAUNCH_CHECK();
    }
    DFTG_MARK(c, "charge");
    return DFTG_OK;
}

// w and w_becke as FP32 hi / lo planes [2][npad] each (once per grid)
__global__ void k_weight_planes(size_t npad, const double *__restrict__ w, const double *__restrict__ wb,
                                float *__restrict__ out)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    const dfl a = df_from(w[p]), b = df_from(wb[p]);
    out[p] = a.h;
    out[npad + p] = a.l;
    out[2 * npad + p] = b.h;
    out[3 * npad + p] = b.l;
}

int launch_weight_planes(dftg_ctx *c)
{
    k_weight_planes<<<(unsigned)((c->npad + 255) / 256), 256, 0, c->stream>>>(c->npad, c->d_w, c->d_wb, c->d_wsplit);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

bool rw_planes(const dftg_ctx *c) { return c->d_rw32 && (c->prec_mask & kPrecMultipole); }

StepLaunch<LdaArgs> step_lda(const dftg_ctx *c, bool apply_scale, bool with_n, bool write_rw)
{
    // with_n: the build's N from the corrected rho (no per-atom sums ran), and
    // (write_rw) the rho w_becke planes for the mixed multipole kernel
    float *rw32 = (with_n && write_rw && rw_planes(c)) ? c->d_rw32 : nullptr;
    const bool mixed = (c->prec_mask & kPrecLda) != 0;
    StepLaunch<LdaArgs> s;
    s.args = LdaArgs{c->npad, c->d_rho, c->d_w, c->d_scal, apply_scale ? 1 : 0,
                     mixed ? ((c->prec_mask & kPrecContract) && c->ct_ready ? 0 : 1) : 1, mixed && with_n ? 1 : 0,
                     c->d_cxc, c->d_cxc32, c->d_red + c->red_lda_off, c->d_counters + kCntLda, mixed ? c->d_wb : nullptr,
                     mixed ? rw32 : nullptr, c->d_wsplit, c->d_wsplit + 2 * c->npad,
                     mixed && cmax_route(c) ? c->d_ct_cmax : nullptr, c->d_ct_winv, c->ct_kbpc * 32};
    s.blocks = (int)((c->npad + kRedBlock - 1) / kRedBlock);
    return s;
}

int launch_xc_points(dftg_ctx *c, bool apply_scale, bool with_n, bool write_rw)
{
    const StepLaunch<LdaArgs> st = step_lda(c, apply_scale, with_n, write_rw);
    if (c->red_lda_off + 2 * (size_t)st.blocks > c->red_elems) {
        set_error("reduction buffer too small for %d blocks", st.blocks);
        return DFTG_ERR_STATE;
    }
    c->rw_ready = st.args.rw32 != nullptr;
    if (c->prec_mask & kPrecLda) DFTG_CUDA(launch_pdl(k_lda<true>, st.blocks, kRedBlock, 0, c->stream, st.args));
    else DFTG_CUDA(launch_pdl(k_lda<false>, st.blocks, kRedBlock, 0, c->stream, st.args));
    DFTG_MARK(c, "lda");
    return DFTG_OK;
}

int group_sums_lda(const SumsArgs *d_sums, const GroupQueue &qs, const LdaArgs *d_lda, const GroupQueue &ql,
                   const SumsLdaCtl &ctl, int nsm, cudaStream_t st)
{
    int occ = 0;
    DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_sums_lda_group, kRedBlock, 0));
    GroupQueue all = ql;
    all.nitems = qs.nitems + ql.nitems;
    const int grid = group_grid(all, occ, nsm);
    if (grid > 0) k_sums_lda_group<<<grid, kRedBlock, 0, st>>>(d_sums, qs, d_lda, ql, ctl);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// partials of the block reductions: two per 256-point block (LDA: E_xc and N;
// E_J: one), one per
// stage-1 chunk of the per-atom sums, two per CTA of the fused density + LDA
// pass (at most one CTA per SM; kMaxRedCtas bounds the SM count)
size_t lda_blocks(size_t npad) { return (npad + kRedBlock - 1) / kRedBlock; }

size_t reduction_elems(size_t npad, int natoms, int nrad, int nang)
{
    size_t a = (npad + kRedBlock - 1) / kRedBlock;
    size_t per_atom = (size_t)nrad * nang;
    size_t b = (size_t)natoms * ((per_atom + kRedChunk - 1) / kRedChunk);
    size_t m = 2 * a > b ? 2 * a : b;      // two partials per block in the point kernel
    return m > 2 * (size_t)kMaxRedCtas ? m : 2 * (size_t)kMaxRedCtas;
}

}  // namespace dftg
