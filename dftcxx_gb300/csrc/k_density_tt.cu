// k_density_tt.cu -- mixed-path density rho_p = 2 phi_p^T P phi_p on the tcgen05
// tensor cores for basis sets of 81 to 1024 functions (gridpoint.cpp:82-84),
// accurate to ~1e-8 relative like the <= 80-function kernel.
//
// T = Phi P as a GEMM over 128-point tiles (M, TMEM lanes) and 128-function
// column blocks nb (N), K = mu in stages of 32 functions:
//   Phi[p, mu] 2^(7 - e_p)  = a_1 + a_2 + a_3 + a_4     (per point e_p)
//   P[mu, nu]  2^(7 - t_nu) = b_1 + b_2 + b_3 + b_4     (per column t_nu)
// a_1 = rint(x) (an integer, |a_1| <= 128), a_2 = bf16(x - a_1), a_3 and a_4 the
// BF16 roundings of what remains (about 31 bits in all), likewise b.  The leading
// products a_1 b_1 are integers <= 2^14, their sum over at most 1024 functions
// (<= 2^24) is exact in the FP32 accumulator D_hi; the nine pairs with
// i + j <= 5 go to D_lo (about 2^-8 of D_hi, FP32 rounding near 2^-32 of it).
// The epilogue forms T = (D_hi + D_lo) 2^(e_p + t_nu - 14) (TwoSum) and
// rho_p = 2 sum_nu T_nu phi_nu in double-float, phi_nu read in FP64 from HBM.
//
// Layouts (canonical no-swizzle K-major core matrices, LBO 128 B, SBO 512 B):
//   A: [tile][K stage][slice][128 points x 32 functions]  (32 KB per stage)
//   B: [nb][K stage][slice][128 columns x 32 functions]   (32 KB per stage)
// CTA persistent over point tiles, each tile over every column block nb:
//   warp 0     loader: two 32 KB bulk copies per stage (A, then B)
//   warp 1     TMEM owner (two buffers of D_hi + D_lo, 512 columns), MMA issuer
//   warps 2-17 epilogue: warp % 4 = TMEM lane quarter (points), (warp - 2) / 4 =
//              its 32 columns; the drain of one block overlaps the MMAs of the
//              next, and the four column groups of a point meet in shared memory
//              after the last block of the tile
// Every mbarrier wait is bounded: on expiry the CTA records an error code, lets
// its copies and MMAs complete, frees TMEM and exits.
#include <cuda_bf16.h>
#include <cstdint>
#include "dftg_internal.cuh"
#include "tc_common.cuh"

namespace dftg {

constexpr int kDtKS = 32;                         // functions (K) per stage
constexpr int kDtKcores = kDtKS / 8;
constexpr int kDtBlk = 128;                       // points per tile = columns per block
constexpr int kDtMinNbf = 81;                     // smaller sets use k_density_tc
constexpr int kDtMaxNbf = 1024;
constexpr int kDtSlices = 4;
constexpr int kDtEpiWarps = 16;
constexpr int kDtThreads = (2 + kDtEpiWarps) * 32;
constexpr int kDtStages = 3;
constexpr uint32_t kDtSlice = kDtBlk * kDtKS * 2;           // 8 KB
constexpr uint32_t kDtHalf = kDtSlices * kDtSlice;          // 32 KB: A or B of one stage
constexpr uint32_t kDtStage = 2 * kDtHalf;
constexpr uint32_t kDtTmemCols = 512;
constexpr int kDtExpMin = -100, kDtExpMax = 100;

struct DtShared {
    uint64_t full[kDtStages], empty[kDtStages];
    uint64_t tmem_full[2], tmem_empty[2], drain;
    uint32_t tmem_base;
    int fail;
    float2 red[4][kDtBlk];                        // per point, the four column groups' sums
};

__device__ __forceinline__ void dt_epi_bar()
{
    asm volatile("bar.sync 1, %0;" ::"n"(kDtEpiWarps * 32) : "memory");
}

// exponent e with m < 2^e (m >= 0), clamped; 0 for m = 0
__device__ __forceinline__ int dt_exp(double m)
{
    int e = 0;
    if (m > 0.0) frexp(m, &e);
    return e < kDtExpMin ? kDtExpMin : (e > kDtExpMax ? kDtExpMax : e);
}

// x (|x| < 128, exact in double) -> four BF16 slices, the first an integer
__device__ __forceinline__ void dt_split4(double x, __nv_bfloat16 (&s)[kDtSlices])
{
    const double a1 = rint(x);
    double r = x - a1;                            // exact
    s[0] = __float2bfloat16_rn((float)a1);        // exact: integer <= 128
#pragma unroll
    for (int i = 1; i < kDtSlices; ++i) {
        s[i] = __float2bfloat16_rn((float)r);
        r -= (double)__bfloat162float(s[i]);      // exact
    }
}

// set-up: e_p = exponent bound of max_mu |phi[p, mu]|, thread per point
__global__ void k_dt_rowexp(int nbf, size_t npad, const double *__restrict__ phi, int *__restrict__ pexp)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    double m = 0.0;
    for (int mu = 0; mu < nbf; ++mu) m = fmax(m, fabs(phi[(size_t)mu * npad + p]));
    pexp[p] = dt_exp(m);
}

// set-up: A slices, thread per (point, 8-function group, K stage, tile), points fastest
__global__ void k_dt_slice_A(int nbf, int nks, size_t npad, const double *__restrict__ phi,
                             const int *__restrict__ pexp, __nv_bfloat16 *__restrict__ A)
{
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t ntile = npad / kDtBlk;
    if (id >= ntile * nks * 4 * kDtBlk) return;
    const int r = (int)(id % kDtBlk);
    const int g = (int)((id / kDtBlk) & 3);
    const int ks = (int)((id / (4 * kDtBlk)) % nks);
    const size_t t = id / ((size_t)4 * kDtBlk * nks);
    const size_t p = t * kDtBlk + r;
    const int e = pexp[p];
    // the eight K values of one core-matrix row: one 16-byte store per slice
    uint32_t w[kDtSlices][4];
#pragma unroll
    for (int k = 0; k < 8; k += 2) {
        const int mu = ks * kDtKS + 8 * g + k;
        const double x0 = mu < nbf ? ldexp(phi[(size_t)mu * npad + p], 7 - e) : 0.0;
        const double x1 = mu + 1 < nbf ? ldexp(phi[(size_t)(mu + 1) * npad + p], 7 - e) : 0.0;
        __nv_bfloat16 s0[kDtSlices], s1[kDtSlices];
        dt_split4(x0, s0);
        dt_split4(x1, s1);
#pragma unroll
        for (int i = 0; i < kDtSlices; ++i)
            w[i][k / 2] = (uint32_t)__bfloat16_as_ushort(s0[i]) | ((uint32_t)__bfloat16_as_ushort(s1[i]) << 16);
    }
    uint4 *dst = reinterpret_cast<uint4 *>(A + ((t * nks + ks) * kDtSlices) * (kDtSlice / 2)) +
                 core_off(r, 8 * g, kDtKcores) / 16;
#pragma unroll
    for (int i = 0; i < kDtSlices; ++i) dst[(size_t)i * (kDtSlice / 16)] = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

// every build: B slices of P and the column exponents, warp per column nu < nnb * 128
__global__ void k_dt_slice_P(int nbf, int nks, int ncol, const double *__restrict__ P, __nv_bfloat16 *__restrict__ B,
                             int *__restrict__ texp)
{
    const int nu = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (nu >= ncol) return;
    double m = 0.0;
    if (nu < nbf)
        for (int mu = lane; mu < nbf; mu += 32) m = fmax(m, fabs(P[(size_t)nu * nbf + mu]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    const int t = dt_exp(m);
    if (lane == 0) texp[nu] = t;
    const int nb = nu / kDtBlk, r = nu % kDtBlk;
    for (int mu = lane; mu < nks * kDtKS; mu += 32) {
        const double y = (nu < nbf && mu < nbf) ? ldexp(P[(size_t)nu * nbf + mu], 7 - t) : 0.0;
        __nv_bfloat16 s[kDtSlices];
        dt_split4(y, s);
        const int ks = mu / kDtKS;
        __nv_bfloat16 *dst = B + (((size_t)nb * nks + ks) * kDtSlices) * (kDtSlice / 2) +
                             core_off(r, mu % kDtKS, kDtKcores) / 2;
#pragma unroll
        for (int i = 0; i < kDtSlices; ++i) dst[(size_t)i * (kDtSlice / 2)] = s[i];
    }
}

__global__ void __launch_bounds__(kDtThreads, 1)
k_density_tt(int nbf, int nks, int nnb, int ntile, size_t npad, const unsigned char *__restrict__ A,
             const unsigned char *__restrict__ B, const int *__restrict__ pexp, const int *__restrict__ texp,
             const double *__restrict__ phi, double *__restrict__ rho, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    DtShared *sh = reinterpret_cast<DtShared *>(smem + (size_t)kDtStages * kDtStage);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nst = kDtStages;

    if (threadIdx.x == 0) {
        for (int s = 0; s < nst; ++s) {
            mbar_init(&sh->full[s], 1);
            mbar_init(&sh->empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sh->tmem_full[b], 1);
            mbar_init(&sh->tmem_empty[b], 1);
        }
        mbar_init(&sh->drain, 1);
        sh->fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(kDtTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;

    if (warp == 0) {
        // ------------------------------------------------------------ loader
        if (lane == 0) {
            int it = 0, issued = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntile && ok; t += gridDim.x)
                for (int nb = 0; nb < nnb && ok; ++nb)
                    for (int ks = 0; ks < nks; ++ks, ++it) {
                        const int s = it % nst, n = it / nst;
                        if (!mbar_wait(&sh->empty[s], (uint32_t)((n & 1) ^ 1)) || sh->fail) {
                            atomicExch(err, 31);
                            sh->fail = 1;
                            ok = false;
                            break;
                        }
                        unsigned char *st = smem + (size_t)s * kDtStage;
                        mbar_arrive_expect_tx(&sh->full[s], kDtStage);
                        bulk_g2s(st, A + ((size_t)t * nks + ks) * kDtHalf, kDtHalf, &sh->full[s]);
                        bulk_g2s(st + kDtHalf, B + ((size_t)nb * nks + ks) * kDtHalf, kDtHalf, &sh->full[s]);
                        issued = it + 1;
                    }
            for (int j = (issued > nst ? issued - nst : 0); j < issued; ++j)
                mbar_wait(&sh->full[j % nst], (uint32_t)((j / nst) & 1));
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(kDtBlk, kDtBlk);
            const uint64_t desc0 = smem_desc(smem, 128, kDtKcores * 128);
            int it = 0, cc = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntile && ok; t += gridDim.x)
                for (int nb = 0; nb < nnb && ok; ++nb, ++cc) {
                    const int buf = cc & 1;
                    if (!mbar_wait(&sh->tmem_empty[buf], (uint32_t)(((cc >> 1) & 1) ^ 1))) {
                        atomicExch(err, 32);
                        sh->fail = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d_hi = tmem + (uint32_t)buf * 256u, d_lo = d_hi + 128u;
                    uint32_t acc_hi = 0, acc_lo = 0;
                    for (int ks = 0; ks < nks; ++ks, ++it) {
                        const int s = it % nst, n = it / nst;
                        if (!mbar_wait(&sh->full[s], (uint32_t)(n & 1)) || sh->fail) {
                            atomicExch(err, 33);
                            sh->fail = 1;
                            ok = false;
                            break;
                        }
                        tc_fence_after();
                        const uint64_t st = desc_add(desc0, (uint32_t)s * kDtStage);
#pragma unroll
                        for (int kk = 0; kk < kDtKS / 16; ++kk) {
                            const uint32_t ko = (uint32_t)kk * 256u;
#pragma unroll
                            for (int i = 0; i < kDtSlices; ++i)
#pragma unroll
                                for (int j = 0; i + j < kDtSlices; ++j) {
                                    const uint64_t ad = desc_add(st, (uint32_t)i * kDtSlice + ko);
                                    const uint64_t bd = desc_add(st, kDtHalf + (uint32_t)j * kDtSlice + ko);
                                    if (i == 0 && j == 0) {
                                        mma_bf16(d_hi, ad, bd, idesc, acc_hi);
                                        acc_hi = 1;
                                    } else {
                                        mma_bf16(d_lo, ad, bd, idesc, acc_lo);
                                        acc_lo = 1;
                                    }
                                }
                        }
                        mma_commit(&sh->empty[s]);
                    }
                    if (!ok) break;
                    mma_commit(&sh->tmem_full[buf]);
                }
            mma_commit(&sh->drain);
            mbar_wait(&sh->drain, 0);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;                   // TMEM lane quarter: points 32 q ..
        const int h = (warp - 2) >> 2;            // columns 32 h .. 32 h + 31 of each block
        const int r = q * 32 + lane;
        int cc = 0;
        bool stop = false;
        for (int t = blockIdx.x; t < ntile && !stop; t += gridDim.x) {
            const size_t p = (size_t)t * kDtBlk + r;
            float S = 0.f, E = 0.f;
            for (int nb = 0; nb < nnb; ++nb, ++cc) {
                const int buf = cc & 1;
                const int nu0 = nb * kDtBlk + 32 * h;
                const int tcol = nu0 + lane < nbf ? texp[nu0 + lane] : 0;   // lane j: column j
                const bool ok = mbar_wait(&sh->tmem_full[buf], (uint32_t)((cc >> 1) & 1));
                if (!ok) {
                    atomicExch(err, 34);
                    sh->fail = 1;
                }
                dt_epi_bar();
                if (sh->fail) {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)buf * 256u + 32u * (uint32_t)h;
#pragma unroll
                for (int b8 = 0; b8 < 4; ++b8) {
                    double f64[8];
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int nu = nu0 + 8 * b8 + k;
                        // streamed once: evict-first, so the A slices of the tile stay in L2
                        f64[k] = nu < nbf ? __ldcs(phi + (size_t)nu * npad + p) : 0.0;
                    }
                    float dh[8], dl[8];
                    tmem_ld8(ta + 8u * b8, dh);
                    tmem_ld8(ta + 128u + 8u * b8, dl);
                    tmem_wait_ld();
#pragma unroll
                    for (int k = 0; k < 8; ++k) {
                        const int j = 8 * b8 + k;
                        const int tc = __shfl_sync(0xffffffffu, tcol, j);
                        // T 2^-e_p = (D_hi + D_lo) 2^(t_nu - 14): exact head by TwoSum
                        const float u = dh[k] + dl[k];
                        const float bp = u - dh[k];
                        float te = (dh[k] - (u - bp)) + (dl[k] - bp);
                        const float sc = __int_as_float((127 - 14 + tc) << 23);   // tc in [-100, 100]
                        const float tv = u * sc;
                        te *= sc;
                        const float fh = (float)f64[k];
                        const float fl = (float)(f64[k] - (double)fh);
                        // S + E += (tv + te)(fh + fl)
                        const float pr = tv * fh;
                        const float pe = fmaf(tv, fh, -pr);
                        const float w = S + pr;
                        const float bq = w - S;
                        E += (S - (w - bq)) + (pr - bq) + pe + fmaf(tv, fl, te * fh);
                        S = w;
                    }
                }
                tc_fence_before();
                dt_epi_bar();                          // TMEM reads of this buffer done
                if (threadIdx.x == 64) mbar_arrive(&sh->tmem_empty[buf]);
            }
            if (stop) break;
            // the four column groups of each point, added in a fixed order
            sh->red[h][r] = make_float2(S, E);
            dt_epi_bar();
            if (h == 0) {
                dfl a{sh->red[0][r].x, sh->red[0][r].y};
#pragma unroll
                for (int g = 1; g < 4; ++g) a = df_add(a, dfl{sh->red[g][r].x, sh->red[g][r].y});
                rho[p] = ldexp(2.0 * df_to(a), pexp[p]);
            }
            dt_epi_bar();
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kDtTmemCols) : "memory");
    }
}

static size_t dt_smem() { return (size_t)kDtStages * kDtStage + sizeof(DtShared); }

int density_tt_setup(dftg_ctx *c)
{
    if (c->nbf < kDtMinNbf || c->nbf > kDtMaxNbf) return DFTG_OK;
    int nsm = 0, optin = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    DFTG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    cudaFuncAttributes fa{};
    DFTG_CUDA(cudaFuncGetAttributes(&fa, k_density_tt));
    if (dt_smem() + fa.sharedSizeBytes > (size_t)optin) return DFTG_OK;
    const int nks = (c->nbf + kDtKS - 1) / kDtKS;
    const int nnb = (c->nbf + kDtBlk - 1) / kDtBlk;
    const size_t ntile = c->npad / kDtBlk;
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density_tt), c->device));
    if (!c->d_flag) {
        DFTG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
    }
    DFTG_CUDA(cudaMalloc(&c->d_dt_A, (size_t)kDtHalf * ntile * nks));
    DFTG_CUDA(cudaMalloc(&c->d_dt_B, (size_t)kDtHalf * nnb * nks));
    DFTG_CUDA(cudaMalloc(&c->d_dt_exp, sizeof(int) * (c->npad + (size_t)nnb * kDtBlk)));
    k_dt_rowexp<<<(unsigned)((c->npad + 255) / 256), 256, 0, c->stream>>>(c->nbf, c->npad, c->d_phi, c->d_dt_exp);
    DFTG_LAUNCH_CHECK();
    const size_t threads = ntile * nks * 4 * kDtBlk;
    k_dt_slice_A<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->nbf, nks, c->npad, c->d_phi, c->d_dt_exp, reinterpret_cast<__nv_bfloat16 *>(c->d_dt_A));
    DFTG_LAUNCH_CHECK();
    c->dt_nks = nks;
    c->dt_nnb = nnb;
    c->dt_grid = (int)(ntile < (size_t)nsm ? ntile : (size_t)nsm);
    c->dt_ready = true;
    return DFTG_OK;
}

int launch_density_tt(dftg_ctx *c)
{
    const int ncol = c->dt_nnb * kDtBlk;
    int *texp = c->d_dt_exp + c->npad;
    k_dt_slice_P<<<(unsigned)((ncol + 7) / 8), 256, 0, c->stream>>>(
        c->nbf, c->dt_nks, ncol, c->d_P, reinterpret_cast<__nv_bfloat16 *>(c->d_dt_B), texp);
    DFTG_LAUNCH_CHECK();
    k_density_tt<<<c->dt_grid, kDtThreads, dt_smem(), c->stream>>>(
        c->nbf, c->dt_nks, c->dt_nnb, (int)(c->npad / kDtBlk), c->npad,
        reinterpret_cast<const unsigned char *>(c->d_dt_A), reinterpret_cast<const unsigned char *>(c->d_dt_B),
        c->d_dt_exp, texp, c->d_phi, c->d_rho, c->d_flag);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

}  // namespace dftg
