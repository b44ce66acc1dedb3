// k_contract_tt.cu -- mixed-path XC or J contraction on the tcgen05 tensor cores
// for basis sets of 129 to 1024 functions (dft.cpp:424-432, atomicgrid.cpp:471-488):
//
//   X = phi^T diag(c) phi,   c = w v_xc (XC) or w V / 2 (J), one pass per matrix
//
// over 128 x 128 tiles (rb, cb), rb <= cb, of the symmetric result, split along
// the points (K):
//   D[m][n] = sum_p B[mu][p] A[nu][p],   mu = 128 rb + m (TMEM lane), nu = 128 cb + n
//   B = c o phi    BF16 slices written by k_tt_build every pass
//   A = phi        BF16 slices written once per grid (the layout and scaling of
//                  the <= 128-function kernel, rows padded to a multiple of 128)
// Number format (per point chunk of at most 512 points): row nu of A is scaled by
// 2^(7 - e_nu) (e_nu: exponent bound of max |phi_nu| over the chunk), row mu of B
// by 2^(7 - s_mu - v) (s_mu: bound of max |w phi_mu|, v: bound of max |c / w|);
// each is split into three BF16 slices, the first an integer of magnitude <= 128,
// so the leading products sum exactly in the FP32 accumulator D_hi within a chunk
// (|sum| < 2^23) and the five correction products go to D_lo.  The epilogue
// scales both back by the exact power of two 2^(s_mu + v + e_nu - 14) and adds
// them to a double-float (FP32 hi + lo, TwoSum) partial held in registers.
//
// Every operand of a stage arrives by bulk copy (no producer warps: B is formed
// in HBM beforehand), so the ring is refilled as soon as the MMAs free a slot.
// CTA = (tile, K part); chunks kp, kp + ksplit, ... of the points.  Warps:
//   warp 0     loader: six bulk copies of 8 KB per stage (3 B slices, 3 A slices)
//   warp 1     TMEM owner (512 columns: two buffers of D_hi + D_lo) and MMA issuer
//   warps 2-17 epilogue: warp % 4 = TMEM lane quarter, (warp - 2) / 4 = its 32
//              columns; the drain of one chunk overlaps the MMAs of the next
// The CTA partial goes to HBM once, at the end; k_contract_tt_reduce adds the K
// parts of each element in a fixed order and symmetrises.  Every mbarrier wait
// is bounded: on expiry the CTA records an error code, lets its copies and MMAs
// complete, frees TMEM and exits.
#include <cuda_bf16.h>
#include <cstdint>
#include "dftg_internal.cuh"
#include "tc_common.cuh"

namespace dftg {

constexpr int kTtKS = 32;                        // points per stage
constexpr int kTtKcores = kTtKS / 8;             // core matrices along K per stage
constexpr int kTtBlk = 128;                      // functions per tile side (M = N = 128)
constexpr int kTtMinNbf = 129;                   // smaller sets use k_contract_tc
constexpr int kTtMaxNbf = 1024;
constexpr int kTtEpiWarps = 16;                  // four per TMEM lane quarter, 32 columns each
constexpr int kTtThreads = (2 + kTtEpiWarps) * 32;
constexpr int kTtStages = 4;
constexpr int kTtMaxKbPerChunk = 16;             // <= 512 points per exact integer accumulation
constexpr uint32_t kTtSlice = kTtBlk * kTtKS * 2;   // one BF16 slice of one 128-row block: 8 KB
constexpr uint32_t kTtStage = 6 * kTtSlice;         // B slices 0-2, then A slices 0-2
constexpr uint32_t kTtTmemCols = 512;               // buffer b: D_hi at 256 b, D_lo at 256 b + 128

struct TtShared {
    uint64_t full[kTtStages];      // operand copies of the stage landed
    uint64_t empty[kTtStages];     // MMAs done with the stage
    uint64_t tmem_full[2];         // accumulator buffer complete for its chunk
    uint64_t tmem_empty[2];        // accumulator buffer drained
    uint64_t drain;
    uint32_t tmem_base;
    int fail;
};

__device__ __forceinline__ float tt_pow2(int k)   // 2^k, k clamped to [-126, 127]
{
    k = k < -126 ? -126 : (k > 127 ? 127 : k);
    return __int_as_float((127 + k) << 23);
}

__device__ __forceinline__ void tt_epi_bar()   // named barrier 1 over the epilogue warps
{
    asm volatile("bar.sync 1, %0;" ::"n"(kTtEpiWarps * 32) : "memory");
}

// (rb, cb) of tile t in the order rb = 0, 1, ...; cb = rb .. nrb - 1
__device__ __forceinline__ int2 tt_tile(int t, int nrb)
{
    int rb = 0;
    while (rb < nrb - 1 && t >= nrb - rb) {
        t -= nrb - rb;
        ++rb;
    }
    return make_int2(rb, rb + t);
}

// B slices of one pass: x = (phi 2^(7 - s_mu)) (c 2^-v), |x| < 128, three BF16
// slices (the first an integer).  Thread per (stage block kb, row < nbf, 8-point
// group g); rows nbf .. AR - 1 stay zero from set-up.
__global__ void __launch_bounds__(256) k_tt_build(int nbf, int AR, size_t npad, int nkb, int kbpc, int which,
                                                  const float *__restrict__ phi, const float *__restrict__ coef,
                                                  const int *__restrict__ swexp, const int2 *__restrict__ cexp,
                                                  uint4 *__restrict__ B)
{
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= (size_t)nkb * nbf * 4) return;
    const int g = (int)(id & 3);
    const int row = (int)((id >> 2) % (size_t)nbf);
    const int kb = (int)(id / ((size_t)nbf * 4));
    const int ch = kb / kbpc;
    const int2 ce = cexp[ch];
    const float fu = tt_pow2(7 - swexp[(size_t)ch * nbf + row]);
    const float fc = tt_pow2(-(which ? ce.y : ce.x));
    const size_t p = (size_t)kb * kTtKS + 8 * g;
    const float4 f0 = *reinterpret_cast<const float4 *>(phi + (size_t)row * npad + p);
    const float4 f1 = *reinterpret_cast<const float4 *>(phi + (size_t)row * npad + p + 4);
    const float4 c0 = *reinterpret_cast<const float4 *>(coef + p);
    const float4 c1 = *reinterpret_cast<const float4 *>(coef + p + 4);
    const float fv[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
    const float cv[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
    uint32_t w[3][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        float x0 = (fv[2 * j] * fu) * (cv[2 * j] * fc);
        float x1 = (fv[2 * j + 1] * fu) * (cv[2 * j + 1] * fc);
        const float i0 = rintf(x0), i1 = rintf(x1);
        const __nv_bfloat162 h1 = __floats2bfloat162_rn(i0, i1);   // exact: integers <= 128
        x0 -= i0;                                                  // exact
        x1 -= i1;
        const __nv_bfloat162 h2 = __floats2bfloat162_rn(x0, x1);
        const float2 f2 = __bfloat1622float2(h2);
        const __nv_bfloat162 h3 = __floats2bfloat162_rn(x0 - f2.x, x1 - f2.y);
        w[0][j] = *reinterpret_cast<const uint32_t *>(&h1);
        w[1][j] = *reinterpret_cast<const uint32_t *>(&h2);
        w[2][j] = *reinterpret_cast<const uint32_t *>(&h3);
    }
    const size_t blk = (size_t)AR * kTtKS * 2 / 16;                 // uint4 per slice block
    const size_t o = core_off(row, 8 * g, kTtKcores) / 16;
#pragma unroll
    for (int i = 0; i < 3; ++i) B[((size_t)kb * 3 + i) * blk + o] = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

__global__ void __launch_bounds__(kTtThreads, 1)
k_contract_tt(int nbf, int AR, int nst, int nkb, int kbpc, int nchunk, int ntiles, int ksplit, int which,
              const unsigned char *__restrict__ bsl, const unsigned char *__restrict__ asl,
              const int *__restrict__ rowexp, const int *__restrict__ swexp, const int2 *__restrict__ cexp,
              float2 *__restrict__ part, int *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    TtShared *sh = reinterpret_cast<TtShared *>(smem + (size_t)nst * kTtStage);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tile = (int)blockIdx.x % ntiles, kp = (int)blockIdx.x / ntiles;
    const int2 tb = tt_tile(tile, AR / kTtBlk);
    const size_t slice_g = (size_t)AR * kTtKS * 2;     // bytes of one slice of one stage block in HBM

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
                     "r"(kTtTmemCols)
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
            for (int ch = kp; ch < nchunk && ok; ch += ksplit) {
                const int kb0 = ch * kbpc, kb1 = min(nkb, kb0 + kbpc);
                for (int kb = kb0; kb < kb1; ++kb, ++it) {
                    const int s = it % nst, n = it / nst;
                    if (!mbar_wait(&sh->empty[s], (uint32_t)((n & 1) ^ 1)) || sh->fail) {
                        atomicExch(err, 21);
                        sh->fail = 1;
                        ok = false;
                        break;
                    }
                    unsigned char *st = smem + (size_t)s * kTtStage;
                    mbar_arrive_expect_tx(&sh->full[s], kTtStage);
                    const size_t base = (size_t)kb * 3 * slice_g;
#pragma unroll
                    for (int i = 0; i < 3; ++i) {
                        bulk_g2s(st + i * kTtSlice, bsl + base + i * slice_g + (size_t)tb.x * kTtSlice, kTtSlice,
                                 &sh->full[s]);
                        bulk_g2s(st + (3 + i) * kTtSlice, asl + base + i * slice_g + (size_t)tb.y * kTtSlice,
                                 kTtSlice, &sh->full[s]);
                    }
                    issued = it + 1;
                }
            }
            // the copies of the last nst stages land before the CTA exits
            for (int j = (issued > nst ? issued - nst : 0); j < issued; ++j)
                mbar_wait(&sh->full[j % nst], (uint32_t)((j / nst) & 1));
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(kTtBlk, kTtBlk);
            const uint64_t desc0 = smem_desc(smem, 128, kTtKcores * 128);
            int it = 0, cc = 0;
            bool ok = true;
            for (int ch = kp; ch < nchunk && ok; ch += ksplit, ++cc) {
                const int buf = cc & 1;
                if (!mbar_wait(&sh->tmem_empty[buf], (uint32_t)(((cc >> 1) & 1) ^ 1))) {
                    atomicExch(err, 22);
                    sh->fail = 1;
                    break;
                }
                tc_fence_after();
                const uint32_t d_hi = tmem + (uint32_t)buf * 256u, d_lo = d_hi + 128u;
                const int kb0 = ch * kbpc, kb1 = min(nkb, kb0 + kbpc);
                uint32_t acc_hi = 0, acc_lo = 0;
                for (int kb = kb0; kb < kb1; ++kb, ++it) {
                    const int s = it % nst, n = it / nst;
                    if (!mbar_wait(&sh->full[s], (uint32_t)(n & 1)) || sh->fail) {
                        atomicExch(err, 23);
                        sh->fail = 1;
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t st = desc_add(desc0, (uint32_t)s * kTtStage);
#pragma unroll
                    for (int kk = 0; kk < kTtKS / 16; ++kk) {
                        const uint32_t ko = (uint32_t)kk * 256u;
#pragma unroll
                        for (int i = 0; i < 3; ++i)
#pragma unroll
                            for (int j = 0; i + j < 3; ++j) {
                                const uint64_t bd = desc_add(st, (uint32_t)i * kTtSlice + ko);
                                const uint64_t ad = desc_add(st, (uint32_t)(3 + j) * kTtSlice + ko);
                                if (i == 0 && j == 0) {
                                    mma_bf16(d_hi, bd, ad, idesc, acc_hi);
                                    acc_hi = 1;
                                } else {
                                    mma_bf16(d_lo, bd, ad, idesc, acc_lo);
                                    acc_lo = 1;
                                }
                            }
                    }
                    mma_commit(&sh->empty[s]);   // the stage is free once these MMAs have read it
                }
                if (!ok) break;
                mma_commit(&sh->tmem_full[buf]);
            }
            // every MMA issued by this thread completes before TMEM is released
            mma_commit(&sh->drain);
            mbar_wait(&sh->drain, 0);
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;                   // TMEM lane quarter of this warp
        const int h = (warp - 2) >> 2;            // columns 32 h .. 32 h + 31
        const int r = q * 32 + lane;              // accumulator row
        const int mu = tb.x * kTtBlk + r;         // B row: basis function
        const int nu0 = tb.y * kTtBlk + 32 * h;   // A row of the first column
        float ps[32], pe[32];                     // double-float partial of the 32 columns
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            ps[j] = 0.f;
            pe[j] = 0.f;
        }
        int cc = 0;
        for (int ch = kp; ch < nchunk; ch += ksplit, ++cc) {
            const int buf = cc & 1;
            // scale exponents: row s_mu + v - 14 (this lane), column e_nu (lane j holds column j)
            const int2 ce = cexp[ch];
            const int erow = mu < nbf ? swexp[(size_t)ch * nbf + mu] + (which ? ce.y : ce.x) - 14 : 0;
            const int ecol = nu0 + lane < nbf ? rowexp[(size_t)ch * nbf + nu0 + lane] : 0;
            const bool ok = mbar_wait(&sh->tmem_full[buf], (uint32_t)((cc >> 1) & 1));
            if (!ok) {
                atomicExch(err, 24);
                sh->fail = 1;
            }
            tt_epi_bar();
            if (sh->fail) break;
            tc_fence_after();
            const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)buf * 256u + 32u * (uint32_t)h;
#pragma unroll
            for (int b8 = 0; b8 < 4; ++b8) {
                float dh[8], dl[8];
                tmem_ld8(ta + 8u * b8, dh);
                tmem_ld8(ta + 128u + 8u * b8, dl);
                tmem_wait_ld();
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    const int j = 8 * b8 + k;
                    const int ec = __shfl_sync(0xffffffffu, ecol, j);
                    const int nu = nu0 + j;
                    // upper triangle only; the factor is an exact power of two
                    const float f = (mu <= nu && nu < nbf) ? tt_pow2(erow + ec) : 0.f;
                    const float vh = dh[k] * f, vl = dl[k] * f;
                    const float t = ps[j] + vh;
                    const float bp = t - ps[j];
                    float e2 = pe[j] + (ps[j] - (t - bp)) + (vh - bp) + vl;
                    const float s2 = t + e2;             // renormalise: |e| <= ulp(s) / 2
                    pe[j] = e2 - (s2 - t);
                    ps[j] = s2;
                }
            }
            tc_fence_before();
            tt_epi_bar();                             // all TMEM reads of this buffer are done
            if (threadIdx.x == 64) mbar_arrive(&sh->tmem_empty[buf]);
        }
        float2 *dst = part + (size_t)blockIdx.x * kTtBlk * kTtBlk;
#pragma unroll
        for (int j = 0; j < 32; ++j) dst[(size_t)(32 * h + j) * kTtBlk + r] = make_float2(ps[j], pe[j]);
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTtTmemCols) : "memory");
    }
}

// Sum the K parts of every element on or above the diagonal in part order
// (double-float), then write it to both triangles of out (column-major).
__global__ void __launch_bounds__(256) k_contract_tt_reduce(int nbf, int nrb, int ntiles, int ksplit,
                                                            const float2 *__restrict__ part, double *__restrict__ out)
{
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (size_t)nbf * nbf) return;
    const int mu = (int)(e % nbf), nu = (int)(e / nbf);
    if (mu > nu) return;
    const int rb = mu / kTtBlk, cb = nu / kTtBlk;
    const int tile = rb * nrb - rb * (rb - 1) / 2 + (cb - rb);
    const size_t off = (size_t)(nu % kTtBlk) * kTtBlk + (mu % kTtBlk);
    dfl s{0.f, 0.f};
    for (int k = 0; k < ksplit; ++k) {
        const float2 a = part[(size_t)(tile + k * ntiles) * kTtBlk * kTtBlk + off];
        s = df_add(s, dfl{a.x, a.y});
    }
    const double v = df_to(s);
    out[(size_t)nu * nbf + mu] = v;
    out[(size_t)mu * nbf + nu] = v;
}

static size_t tt_smem(int nst) { return (size_t)nst * kTtStage + sizeof(TtShared); }

int contract_tt_setup(dftg_ctx *c)
{
    if (c->nbf < kTtMinNbf || c->nbf > kTtMaxNbf) return DFTG_OK;
    int nsm = 0, optin = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    DFTG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    cudaFuncAttributes fa{};
    DFTG_CUDA(cudaFuncGetAttributes(&fa, k_contract_tt));
    if (tt_smem(kTtStages) + fa.sharedSizeBytes > (size_t)optin) return DFTG_OK;
    const int AR = (c->nbf + kTtBlk - 1) / kTtBlk * kTtBlk, nrb = AR / kTtBlk;
    const int ntiles = nrb * (nrb + 1) / 2;
    const int nkb = (int)(c->npad / kTtKS);
    int ksplit = nsm / ntiles;
    if (ksplit < 1) ksplit = 1;
    if (ksplit > nkb) ksplit = nkb;
    // chunks of at most kTtMaxKbPerChunk stages, as even as possible over the K parts
    const int per_kp = (nkb + ksplit * kTtMaxKbPerChunk - 1) / (ksplit * kTtMaxKbPerChunk);
    const int target = ksplit * (per_kp > 0 ? per_kp : 1);
    int kbpc = (nkb + target - 1) / target;
    if (kbpc < 1) kbpc = 1;
    const int nchunk = (nkb + kbpc - 1) / kbpc;
    const int grid = ntiles * ksplit;
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_contract_tt), c->device));
    if (!c->d_flag) {
        DFTG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
    }
    const size_t slices = (size_t)nkb * 3 * AR * kTtKS;   // BF16 elements of one operand
    DFTG_CUDA(cudaMalloc(&c->d_tt_exp, sizeof(int) * 2 * (size_t)nchunk * c->nbf + sizeof(int2) * (size_t)nchunk));
    DFTG_CUDA(cudaMalloc(&c->d_tt_winv, sizeof(float) * c->npad));
    DFTG_CUDA(cudaMalloc(&c->d_tt_A, sizeof(__nv_bfloat16) * slices));
    DFTG_CUDA(cudaMalloc(&c->d_tt_B, sizeof(__nv_bfloat16) * slices));
    DFTG_CUDA(cudaMalloc(&c->d_tt_part, sizeof(float2) * (size_t)grid * kTtBlk * kTtBlk));
    DFTG_CUDA(cudaMemsetAsync(c->d_tt_B, 0, sizeof(__nv_bfloat16) * slices, c->stream));   // rows >= nbf
    DFTG_TRY_L(ct_setup_tables(c, AR, nkb, kbpc, nchunk, c->d_tt_exp, c->d_tt_exp + (size_t)nchunk * c->nbf,
                               c->d_tt_winv, c->d_tt_A));
    c->tt_AR = AR;
    c->tt_nkb = nkb;
    c->tt_kbpc = kbpc;
    c->tt_nchunk = nchunk;
    c->tt_ntiles = ntiles;
    c->tt_ksplit = ksplit;
    c->tt_grid = grid;
    c->tt_ready = true;
    return DFTG_OK;
}

static int2 *tt_cexp(dftg_ctx *c) { return reinterpret_cast<int2 *>(c->d_tt_exp + 2 * (size_t)c->tt_nchunk * c->nbf); }

// per-chunk bounds of |cx / w| and |cy / w| for the passes that follow
int launch_contract_tt_bounds(dftg_ctx *c, const float *cx, const float *cy)
{
    return ct_launch_cexp(c, c->tt_nkb, c->tt_kbpc, c->tt_nchunk, cx, cy, c->d_tt_winv, tt_cexp(c));
}

// out = phi^T diag(coef) phi (nbf x nbf, column-major, FP64); which = 0 / 1 picks
// the bound of coef among the two of the preceding launch_contract_tt_bounds
int launch_contract_tt(dftg_ctx *c, const float *coef, int which, double *out)
{
    const int *rowexp = c->d_tt_exp, *swexp = c->d_tt_exp + (size_t)c->tt_nchunk * c->nbf;
    const size_t threads = (size_t)c->tt_nkb * c->nbf * 4;
    k_tt_build<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->nbf, c->tt_AR, c->npad, c->tt_nkb, c->tt_kbpc, which, c->d_phi32, coef, swexp, tt_cexp(c),
        reinterpret_cast<uint4 *>(c->d_tt_B));
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "contract_operand");
    k_contract_tt<<<c->tt_grid, kTtThreads, tt_smem(kTtStages), c->stream>>>(
        c->nbf, c->tt_AR, kTtStages, c->tt_nkb, c->tt_kbpc, c->tt_nchunk, c->tt_ntiles, c->tt_ksplit, which,
        reinterpret_cast<const unsigned char *>(c->d_tt_B), reinterpret_cast<const unsigned char *>(c->d_tt_A), rowexp,
        swexp, tt_cexp(c), reinterpret_cast<float2 *>(c->d_tt_part), c->d_flag);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "contract");
    const size_t nn = (size_t)c->nbf * c->nbf;
    k_contract_tt_reduce<<<(unsigned)((nn + 255) / 256), 256, 0, c->stream>>>(
        c->nbf, c->tt_AR / kTtBlk, c->tt_ntiles, c->tt_ksplit, reinterpret_cast<const float2 *>(c->d_tt_part), out);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "contract_reduce");
    return DFTG_OK;
}

}  // namespace dftg
