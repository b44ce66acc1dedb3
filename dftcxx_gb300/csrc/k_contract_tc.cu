// k_contract_tc.cu -- mixed-path XC and J contractions on the tcgen05 tensor cores
// (dft.cpp:424-432, atomicgrid.cpp:471-488):
//
//   XC = phi^T diag(c_xc) phi,   J = phi^T diag(c_j) phi,   c_xc = w v_xc, c_j = w V / 2
//
// as one GEMM per point chunk, D[mu][n] = sum_p A[mu][p] B[n][p], with
//   A = phi (rows mu < nbf of M = 128),
//   B = [c_xc o phi ; c_j o phi] (rows n < 2 nbf of N = NP, NP = 2 nbf rounded up to 16),
// K = points.  Both operands are split into NS BF16 slices, x = x_1 + x_2 (+ x_3),
// x_{i+1} = bf16(x - x_1 - ... - x_i), so the FP32 inputs are carried to 16 (NS = 2)
// or 24 (NS = 3) bits.  The products are accumulated in two TMEM accumulators:
//   D_hi = A_1 B_1                          (the leading term)
//   D_lo = A_1 B_2 + A_2 B_1 (+ A_1 B_3 + A_2 B_2 + A_3 B_1)
// so the rounding of the small terms is not charged to the leading sum.  The point
// dimension is cut into nchunk chunks; each chunk's D_hi + D_lo is written as an
// FP64 partial and the partials are summed in a fixed order by k_contract_reduce,
// which also symmetrises the result.
//
// CTA (persistent over chunks): warps 0-3 produce operand stages from the FP32
// amplitudes and point coefficients (coalesced loads, BF16 slicing, canonical
// no-swizzle K-major core matrices in shared memory, then a proxy fence); warp 4
// owns TMEM and issues the MMAs from one thread; warps 5-8 drain the accumulators.
// Every mbarrier wait is bounded: on expiry the CTA records an error code, lets
// its MMAs complete, frees TMEM and exits.
#include <cuda_bf16.h>
#include <cstdint>
#include "dftg_internal.cuh"
#include "tc_common.cuh"

namespace dftg {

constexpr int kCtKS = 32;                  // points per stage
constexpr int kCtKcores = kCtKS / 8;       // core matrices along K per stage
constexpr int kCtM = 128;
constexpr int kCtMaxNbf = 128;             // 2 nbf <= 256 columns per accumulator
constexpr int kCtThreads = 288;
constexpr int kCtMaxStages = 8;
constexpr int kCtMaxKbPerChunk = 32;       // at most 1024 points per FP32 accumulation
constexpr uint32_t kCtTmemCols = 512;      // D_hi at column 0, D_lo at column 256
constexpr int kCtSlices = 3;

struct CtShared {
    uint64_t full[kCtMaxStages], empty[kCtMaxStages];
    uint64_t tmem_full, tmem_empty, drain;
    uint32_t tmem_base;
    int fail;
};

__device__ __forceinline__ void ct_epi_bar()
{
    asm volatile("bar.sync 1, 128;" ::: "memory");
}

// eight consecutive K values -> NS packed BF16 slices (16 bytes each)
template <int NS>
__device__ __forceinline__ void slice8(const float (&v)[8], uint4 (&out)[NS])
{
    uint32_t w[NS][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float x0 = v[2 * j], x1 = v[2 * j + 1];
#pragma unroll
        for (int i = 0; i < NS; ++i) {
            const __nv_bfloat162 h = __floats2bfloat162_rn(x0, x1);   // .x (low half) = x0
            w[i][j] = *reinterpret_cast<const uint32_t *>(&h);
            if (i + 1 < NS) {
                const float2 f = __bfloat1622float2(h);
                x0 -= f.x;                                             // exact in FP32
                x1 -= f.y;
            }
        }
    }
#pragma unroll
    for (int i = 0; i < NS; ++i) out[i] = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

__host__ __device__ constexpr uint32_t ct_a_slice_bytes() { return (uint32_t)kCtM * kCtKS * 2; }
__host__ __device__ constexpr uint32_t ct_b_slice_bytes(int NP) { return (uint32_t)NP * kCtKS * 2; }
__host__ __device__ constexpr uint32_t ct_stage_bytes(int NS, int NP)
{
    return (uint32_t)NS * (ct_a_slice_bytes() + ct_b_slice_bytes(NP));
}

template <int NS>
__global__ void __launch_bounds__(kCtThreads, 1)
k_contract_tc(int nbf, int NP, int nst, int nkb, int kb_per_chunk, int nchunk, size_t npad,
              const float *__restrict__ phi, const float *__restrict__ cxc, const float *__restrict__ cj,
              double *__restrict__ part, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const uint32_t a_slice = ct_a_slice_bytes(), b_slice = ct_b_slice_bytes(NP);
    const uint32_t stage = ct_stage_bytes(NS, NP);
    CtShared *sh = reinterpret_cast<CtShared *>(smem + (size_t)nst * stage);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // zero the operand stages once: rows >= nbf of A and >= 2 nbf of B are never written
    {
        uint4 *z = reinterpret_cast<uint4 *>(smem);
        const int n16 = (int)((size_t)nst * stage / 16);
        for (int i = threadIdx.x; i < n16; i += kCtThreads) z[i] = make_uint4(0u, 0u, 0u, 0u);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < nst; ++s) {
            mbar_init(&sh->full[s], 1);          // the producing warp
            mbar_init(&sh->empty[s], 1);         // MMA commit
        }
        mbar_init(&sh->tmem_full, 1);
        mbar_init(&sh->tmem_empty, 1);
        mbar_init(&sh->drain, 1);
        sh->fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 4) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(kCtTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh->tmem_base;

    if (warp < 4) {
        // ------------------------------------------------------------ producers
        // warp w fills stages w, w + 4, ... of this CTA's sequence, so four
        // stages are in preparation at once; lane = (row group of 8 mu) x (8-point group g)
        const int g = lane & 3, mrow = lane >> 2;
        int it = 0;
        bool ok = true;
        for (int ch = blockIdx.x; ch < nchunk && ok; ch += gridDim.x) {
            const int kb0 = ch * kb_per_chunk, kb1 = min(nkb, kb0 + kb_per_chunk);
            for (int kb = kb0; kb < kb1; ++kb, ++it) {
                if ((it & 3) != warp) continue;
                const int s = it % nst, n = it / nst;
                int w_ok = 1;
                if (lane == 0) w_ok = mbar_wait(&sh->empty[s], (uint32_t)((n & 1) ^ 1)) ? 1 : 0;
                w_ok = __shfl_sync(0xffffffffu, w_ok, 0);
                if (!w_ok || sh->fail) {
                    if (lane == 0 && !w_ok) { atomicExch(err, 11); sh->fail = 1; }
                    ok = false;
                    break;
                }
                const size_t p = (size_t)kb * kCtKS + 8 * g;
                const float4 x0 = *reinterpret_cast<const float4 *>(cxc + p);
                const float4 x1 = *reinterpret_cast<const float4 *>(cxc + p + 4);
                const float4 j0 = *reinterpret_cast<const float4 *>(cj + p);
                const float4 j1 = *reinterpret_cast<const float4 *>(cj + p + 4);
                const float cx[8] = {x0.x, x0.y, x0.z, x0.w, x1.x, x1.y, x1.z, x1.w};
                const float cy[8] = {j0.x, j0.y, j0.z, j0.w, j1.x, j1.y, j1.z, j1.w};
                unsigned char *sA = smem + (size_t)s * stage;
                unsigned char *sB = sA + NS * a_slice;
                constexpr int U = 3;
                for (int base = 0; base < nbf; base += 8 * U) {
                    float4 f[U][2];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int mu = base + 8 * u + mrow;
                        if (mu < nbf) {
                            f[u][0] = *reinterpret_cast<const float4 *>(phi + (size_t)mu * npad + p);
                            f[u][1] = *reinterpret_cast<const float4 *>(phi + (size_t)mu * npad + p + 4);
                        } else {
                            f[u][0] = make_float4(0.f, 0.f, 0.f, 0.f);
                            f[u][1] = f[u][0];
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const int mu = base + 8 * u + mrow;
                        if (mu >= nbf) continue;
                        const float v[8] = {f[u][0].x, f[u][0].y, f[u][0].z, f[u][0].w,
                                            f[u][1].x, f[u][1].y, f[u][1].z, f[u][1].w};
                        float bx[8], by[8];
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            bx[k] = cx[k] * v[k];
                            by[k] = cy[k] * v[k];
                        }
                        uint4 sa[NS], sbx[NS], sby[NS];
                        slice8<NS>(v, sa);
                        slice8<NS>(bx, sbx);
                        slice8<NS>(by, sby);
                        const uint32_t oa = core_off(mu, 8 * g, kCtKcores);
                        const uint32_t oj = core_off(nbf + mu, 8 * g, kCtKcores);
#pragma unroll
                        for (int i = 0; i < NS; ++i) {
                            *reinterpret_cast<uint4 *>(sA + i * a_slice + oa) = sa[i];
                            *reinterpret_cast<uint4 *>(sB + i * b_slice + oa) = sbx[i];
                            *reinterpret_cast<uint4 *>(sB + i * b_slice + oj) = sby[i];
                        }
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&sh->full[s]);
            }
        }
    } else if (warp == 4) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(kCtM, NP);
            const uint32_t lbo = 128, sbo = kCtKcores * 128;
            const uint32_t d_hi = tmem, d_lo = tmem + 256;
            int it = 0, cc = 0;
            bool ok = true;
            for (int ch = blockIdx.x; ch < nchunk && ok; ch += gridDim.x, ++cc) {
                if (!mbar_wait(&sh->tmem_empty, (uint32_t)((cc & 1) ^ 1))) { atomicExch(err, 12); sh->fail = 1; break; }
                tc_fence_after();
                const int kb0 = ch * kb_per_chunk, kb1 = min(nkb, kb0 + kb_per_chunk);
                uint32_t acc_hi = 0, acc_lo = 0;
                for (int kb = kb0; kb < kb1; ++kb, ++it) {
                    const int s = it % nst, n = it / nst;
                    if (!mbar_wait(&sh->full[s], (uint32_t)(n & 1)) || sh->fail) {
                        atomicExch(err, 13);
                        sh->fail = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const unsigned char *sA = smem + (size_t)s * stage;
                    const unsigned char *sB = sA + NS * a_slice;
#pragma unroll
                    for (int kk = 0; kk < kCtKS / 16; ++kk) {
                        const uint32_t ko = (uint32_t)kk * 2 * lbo;
#pragma unroll
                        for (int i = 0; i < NS; ++i)
#pragma unroll
                            for (int j = 0; i + j < NS; ++j) {
                                const uint64_t ad = smem_desc(sA + i * a_slice + ko, lbo, sbo);
                                const uint64_t bd = smem_desc(sB + j * b_slice + ko, lbo, sbo);
                                if (i == 0 && j == 0) {
                                    mma_bf16(d_hi, ad, bd, idesc, acc_hi);
                                    acc_hi = 1;
                                } else {
                                    mma_bf16(d_lo, ad, bd, idesc, acc_lo);
                                    acc_lo = 1;
                                }
                            }
                    }
                    mma_commit(&sh->empty[s]);   // stage s is free once these MMAs have read it
                }
                if (!ok) break;
                mma_commit(&sh->tmem_full);
            }
            // every MMA issued by this thread completes before TMEM is released
            mma_commit(&sh->drain);
            mbar_wait(&sh->drain, 0);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;                  // TMEM lane quarter of this warp
        const int r = q * 32 + lane;             // accumulator row = basis function mu
        const size_t nn = (size_t)nbf * nbf;
        int cc = 0;
        for (int ch = blockIdx.x; ch < nchunk; ch += gridDim.x, ++cc) {
            const bool ok = mbar_wait(&sh->tmem_full, (uint32_t)(cc & 1));
            if (!ok) { atomicExch(err, 14); sh->fail = 1; }
            ct_epi_bar();
            if (sh->fail) break;
            tc_fence_after();
            const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16);
            double *px = part + (size_t)ch * 2 * nn;
            for (int c0 = 0; c0 < NP; c0 += 16) {
                float dh[16], dl[16];
                tmem_ld16(ta + (uint32_t)c0, dh);
                tmem_ld16(ta + 256u + (uint32_t)c0, dl);
                tmem_wait_ld();
                if (r < nbf) {
#pragma unroll
                    for (int k = 0; k < 16; ++k) {
                        const int nu = c0 + k;
                        const double v = (double)dh[k] + (double)dl[k];
                        if (nu < nbf) px[(size_t)nu * nbf + r] = v;
                        else if (nu < 2 * nbf) px[nn + (size_t)(nu - nbf) * nbf + r] = v;
                    }
                }
            }
            tc_fence_before();
            ct_epi_bar();                        // all TMEM reads of this chunk are done
            if (threadIdx.x == 160) mbar_arrive(&sh->tmem_empty);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCtTmemCols) : "memory");
    }
}

// ------------------------------------------------------------------ host side

static size_t ct_smem(int nst, int NP) { return (size_t)nst * ct_stage_bytes(kCtSlices, NP) + sizeof(CtShared); }

// chunking of the point dimension for nsm CTAs: chunks per CTA is the smallest
// count that keeps every chunk at most kCtMaxKbPerChunk stages long
static void ct_plan(size_t npad, int nsm, int &nkb, int &kbpc, int &nchunk)
{
    nkb = (int)(npad / kCtKS);
    const int per_cta = (nkb + nsm * kCtMaxKbPerChunk - 1) / (nsm * kCtMaxKbPerChunk);
    int target = nsm * (per_cta > 0 ? per_cta : 1);
    kbpc = (nkb + target - 1) / target;
    if (kbpc < 1) kbpc = 1;
    nchunk = (nkb + kbpc - 1) / kbpc;
}

size_t contract_tc_part_elems(int nbf, size_t npad, int nsm)
{
    if (nbf > kCtMaxNbf) return 0;
    int nkb, kbpc, nchunk;
    ct_plan(npad, nsm, nkb, kbpc, nchunk);
    return (size_t)nchunk * 2 * nbf * nbf;
}

int contract_tc_setup(dftg_ctx *c)
{
    if (c->nbf > kCtMaxNbf) return DFTG_OK;
    int nsm = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    int optin = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const int NP = (2 * c->nbf + 15) / 16 * 16;
    int nst = kCtMaxStages;
    while (nst > 2 && ct_smem(nst, NP) > (size_t)optin) --nst;
    if (ct_smem(nst, NP) > (size_t)optin) return DFTG_OK;
    int nkb, kbpc, nchunk;
    ct_plan(c->npad, nsm, nkb, kbpc, nchunk);
    if ((size_t)nchunk * 2 * c->nbf * c->nbf > c->part_elems) return DFTG_OK;
    DFTG_CUDA(cudaFuncSetAttribute(k_contract_tc<kCtSlices>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)ct_smem(nst, NP)));
    if (!c->d_flag) {
        DFTG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
    }
    c->ct_NP = NP;
    c->ct_nst = nst;
    c->ct_nkb = nkb;
    c->ct_kbpc = kbpc;
    c->ct_nchunk = nchunk;
    c->ct_grid = nchunk < nsm ? nchunk : nsm;
    c->ct_ready = true;
    return DFTG_OK;
}

int launch_contract_tc(dftg_ctx *c)
{
    k_contract_tc<kCtSlices><<<c->ct_grid, kCtThreads, ct_smem(c->ct_nst, c->ct_NP), c->stream>>>(
        c->nbf, c->ct_NP, c->ct_nst, c->ct_nkb, c->ct_kbpc, c->ct_nchunk, c->npad, c->d_phi32, c->d_cxc32, c->d_cj32,
        c->d_part, c->d_flag);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

}  // namespace dftg
