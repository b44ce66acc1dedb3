// k_contract_tc.cu -- mixed-path XC and J contractions on the tcgen05 tensor cores
// (dft.cpp:424-432, atomicgrid.cpp:471-488):
//
//   XC = phi^T diag(c_xc) phi,   J = phi^T diag(c_j) phi,   c_xc = w v_xc, c_j = w V / 2
//
// as one GEMM per point chunk, D[mu][n] = sum_p A[mu][p] B[n][p], K = points:
//   A = phi                         rows mu < nbf of M = 128
//   B = [c_xc o phi ; c_j o phi]    rows n < 2 nbf of N = NP (2 nbf rounded up to 16)
//
// Number format (per point chunk of at most 1024 points).  Row mu of A is scaled
// by 2^(7 - e_mu), e_mu the exponent bound of max |phi_mu| over the chunk, and
// split into three BF16 slices: a_1 = rint(x) (an integer, |a_1| <= 128),
// a_2 = bf16(x - a_1), a_3 = bf16(x - a_1 - a_2).  B row nu is scaled by
// 2^(7 - s_nu - v), s_nu the bound of max |w phi_nu| over the chunk (fixed for
// the grid) and v the bound of max |c / w| (per build), and split likewise.  The
// leading products a_1 b_1 are integers of magnitude at most 2^14, so every
// partial sum over a chunk is an integer of magnitude at most 2^24, exact in the
// FP32 accumulator whatever the accumulator's
// rounding; the five correction products (a_1 b_2, a_2 b_1, a_1 b_3, a_2 b_2,
// a_3 b_1) go to a second accumulator, about 2^-8 of the first.  The epilogue
// scales D_hi and D_lo back by exact powers of two and adds them to the CTA's
// partial, a double-float (FP32 hi + lo, TwoSum) matrix in shared memory, so
// no FP64 arithmetic (slow on this GPU) runs per chunk; k_contract_tc_reduce
// sums the CTA partials in FP64 in a fixed order and symmetrises.  A (phi is fixed for the grid) is sliced once at setup into HBM
// in the shared-memory operand layout; B is formed every build from A and c.
//
// CTA (persistent over chunks, 832 threads):
//   warps 0-11  producers in two groups of six: group g builds the B slices of
//               the stages in ring slots of parity g (the ring depth is even, so
//               a group sees each of its slots' phases in order), every warp of
//               the group its rows (w, w + 6, ... in groups of eight), from the A
//               slices and c values of the stage (shared memory), then a proxy
//               fence and an mbarrier arrive (the full barrier counts six);
//   warp 12     TMEM owner and MMA issuer (one thread);
//   warps 13-24 epilogue: TMEM -> double-float partial (TMEM lane quarter =
//               warp % 4, the three warps of a quarter take every third
//               16-column block);
//   warp 25     loader: bulk copies of the A slices and c values of each stage.
// Every mbarrier wait is bounded: on expiry the CTA records an error code, lets
// its copies and MMAs complete, frees TMEM and exits.
#include <cuda_bf16.h>
#include <cstdint>
#include "dftg_internal.cuh"
#include "tc_common.cuh"

namespace dftg {

constexpr int kCtKS = 32;                  // points per stage
constexpr int kCtKcores = kCtKS / 8;       // core matrices along K per stage
constexpr int kCtM = 128;
constexpr int kCtMaxNbf = 128;             // 2 nbf <= 256 columns per accumulator
constexpr int kCtProducers = 12;          // producer warps 0..11, two groups of six
constexpr int kCtGroupWarps = kCtProducers / 2;
constexpr int kCtRowSteps = (kCtMaxNbf + 8 * kCtGroupWarps - 1) / (8 * kCtGroupWarps);   // rows per lane
constexpr int kCtMmaWarp = kCtProducers;   // TMEM owner and MMA issuer
constexpr int kCtEpi0 = kCtMmaWarp + 1;    // epilogue warps kCtEpi0 .. kCtEpi0 + kCtEpiWarps - 1
constexpr int kCtEpiWarps = 12;           // three per TMEM lane quarter
constexpr int kCtThreads = (kCtEpi0 + kCtEpiWarps + 1) * 32;
constexpr int kCtLoaderWarp = kCtEpi0 + kCtEpiWarps;
constexpr int kCtMaxStages = 8;
constexpr int kCtMaxKbPerChunk = 32;       // <= 1024 points per exact integer accumulation (|sums| <= 2^24)
constexpr uint32_t kCtTmemCols = 512;      // D_hi at column 0, D_lo at column 256
constexpr int kCtSlices = 3;
constexpr int kCtExpMin = -100;            // exponent bounds are clamped to [-100, 100]
constexpr int kCtExpMax = 100;

struct CtShared {
    uint64_t a_full[kCtMaxStages];         // A slices and c values landed (bulk copies)
    uint64_t full[kCtMaxStages];           // B slices written (producer warp)
    uint64_t empty[kCtMaxStages];          // MMAs done with the stage
    uint64_t tmem_full, tmem_empty, drain;
    uint32_t tmem_base;
    int fail;
    int item;                              // the grouped launch's queue position (broadcast)
};

__device__ __forceinline__ void ct_epi_bar()   // named barrier 1 over the epilogue warps
{
    asm volatile("bar.sync 1, %0;" ::"n"(kCtEpiWarps * 32) : "memory");
}

__device__ __forceinline__ float pow2f(int k)   // 2^k, -126 <= k <= 127
{
    return __int_as_float((127 + k) << 23);
}

// exponent e with |x| < 2^e for the largest |x| given as FP32 bits, clamped
__device__ __forceinline__ int exp_bound(uint32_t absbits)
{
    const int e = (int)(absbits >> 23) - 126;
    return e < kCtExpMin ? kCtExpMin : (e > kCtExpMax ? kCtExpMax : e);
}

// eight consecutive K values as four packed pairs (scaled, |x| < 128) -> three
// BF16 slices, the first an integer
__device__ __forceinline__ void slice8_fixed(const float2 (&v)[4], uint4 (&out)[kCtSlices])
{
    // rint by the shift 1.5 * 2^23: for |x| < 2^22 the FP32 sums x + 1.5 * 2^23 are
    // spaced by one, so the round-to-nearest-even add rounds x to an integer as
    // rintf does (a packed add and subtract per pair in place of two rounding
    // conversions; the byte permute below replaces the leading slice's conversion)
    const float2 kRint = make_float2(12582912.f, 12582912.f);
    uint32_t w[kCtSlices][4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        // i = +0 where rintf gives -0 (x from -0.5 to -0): the MMA's sums are not
        // invariant to the sign of a zero operand, so the results differ from the
        // rintf form in the last bits of the correction accumulator
        const float2 i = f2sub(f2add(v[j], kRint), kRint);
        const float2 x = f2sub(v[j], i);                           // exact
        const __nv_bfloat162 h2 = __float22bfloat162_rn(x);
        const __nv_bfloat162 h3 = __float22bfloat162_rn(f2sub(x, __bfloat1622float2(h2)));
        // integers of magnitude <= 128 have at most eight significant bits, so their
        // BF16 encodings are the high halves of their FP32 encodings
        w[0][j] = __byte_perm(__float_as_uint(i.x), __float_as_uint(i.y), 0x7632);
        w[1][j] = *reinterpret_cast<const uint32_t *>(&h2);
        w[2][j] = *reinterpret_cast<const uint32_t *>(&h3);
    }
#pragma unroll
    for (int i = 0; i < kCtSlices; ++i) out[i] = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
}

// eight BF16 values (16 bytes) -> four packed FP32 pairs
__device__ __forceinline__ void unpack8(uint4 u, float2 (&v)[4])
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) v[j] = make_float2(__uint_as_float(w[j] << 16), __uint_as_float(w[j] & 0xffff0000u));
}

// per chunk: exponent bounds of max |c_xc / w| and max |c_j / w| (block per chunk)
__device__ __forceinline__ void ct_cexp_block(const CexpArgs A, int ch)
{
    const int nkb = A.nkb, kb_per_chunk = A.kbpc;
    const float *__restrict__ cxc = A.cxc, *__restrict__ cj = A.cj, *__restrict__ winv = A.winv;
    int2 *__restrict__ cexp = A.cexp;
    __shared__ float sx[8], sj[8];
    const size_t p0 = (size_t)ch * kb_per_chunk * kCtKS;
    const size_t p1 = (size_t)min(nkb, (ch + 1) * kb_per_chunk) * kCtKS;
    float mx = 0.f, mj = 0.f;
    for (size_t p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
        const float u = winv[p];
        mx = fmaxf(mx, fabsf(cxc[p]) * u);
        mj = fmaxf(mj, fabsf(cj[p]) * u);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        mj = fmaxf(mj, __shfl_xor_sync(0xffffffffu, mj, o));
    }
    if ((threadIdx.x & 31) == 0) {
        sx[threadIdx.x >> 5] = mx;
        sj[threadIdx.x >> 5] = mj;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
            mx = fmaxf(mx, sx[w]);
            mj = fmaxf(mj, sj[w]);
        }
        cexp[ch] = make_int2(exp_bound(__float_as_uint(mx)), exp_bound(__float_as_uint(mj)));
    }
}

constexpr int kCexpThreads = 256;

__global__ void __launch_bounds__(kCexpThreads) k_ct_cexp(const CexpArgs a) { ct_cexp_block(a, (int)blockIdx.x); }

__global__ void __launch_bounds__(kCexpThreads) k_ct_cexp_group(const CexpArgs *__restrict__ args, GroupQueue q)
{
    __shared__ int s_item;
    gq_run(q, &s_item, [&](int m, int vb, int) {
        const CexpArgs a = args[m];
        ct_cexp_block(a, vb);
        return true;
    });
}

// Stage layout in shared memory: the three A slices packed at a stride of AR
// rows (AR = nbf rounded up to 8) -- the MMA reads 128 rows from each slice
// start, and rows >= AR (the next slice, or the tail) only feed accumulator
// rows >= nbf, which are never read -- then the three B slices of NP rows,
// then c_xc[32] and c_j[32].
__host__ __device__ constexpr uint32_t ct_a_slice_bytes(int AR) { return (uint32_t)AR * kCtKS * 2; }
__host__ __device__ constexpr uint32_t ct_a_region_bytes(int AR)
{
    return (uint32_t)(kCtSlices - 1) * ct_a_slice_bytes(AR) + (uint32_t)kCtM * kCtKS * 2;
}
__host__ __device__ constexpr uint32_t ct_b_slice_bytes(int NP) { return (uint32_t)NP * kCtKS * 2; }
__host__ __device__ constexpr uint32_t ct_stage_bytes(int NP, int AR)
{
    return ct_a_region_bytes(AR) + (uint32_t)kCtSlices * ct_b_slice_bytes(NP) + 2 * kCtKS * 4;
}

// One CTA's share of one molecule's chunks (vb, vb + nvb, ...): zeroes the
// operand stages, initialises the mbarriers, runs the roles and invalidates the
// mbarriers again; the caller owns the kCtTmemCols TMEM columns at tmem.
// Returns false (block-uniform) when a bounded wait gave up.
// the CTA's mbarriers and TMEM address (one instance in every kernel that uses them)
__shared__ CtShared ct_sh;

// G: a grouped launch's item (vb, nvb given); else the CTA of a single launch
// (vb, nvb read from blockIdx / gridDim where used, so they hold no registers)
template <bool G>
__device__ __forceinline__ bool contract_tc_cta(const CtArgs A, int vb_, int nvb_, uint32_t tmem)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    CtShared *sh = &ct_sh;
    const int nbf = A.nbf, AR = A.AR, NP = A.NP, nst = A.nst, spart = A.spart, nkb = A.nkb;
    const int kb_per_chunk = A.kbpc, nchunk = A.nchunk;
    const unsigned char *__restrict__ aslices = A.aslices;
    const int *__restrict__ rowexp = A.rowexp, *__restrict__ swexp = A.swexp;
    const int2 *__restrict__ cexp = A.cexp;
    const unsigned *__restrict__ cmax = A.cmax;
    // exponent bounds of max |c_xc / w| and max |c_j / w| over chunk ch: from the
    // bounds pass, or from the chunk maxima the point kernel and the gather kept
    auto chunk_bounds = [&](int ch) {
        return cmax ? make_int2(exp_bound(cmax[ch]), exp_bound(cmax[nchunk + ch])) : cexp[ch];
    };
    const float *__restrict__ cxc = A.cxc, *__restrict__ cj = A.cj;
    float2 *__restrict__ part = A.part;
    int *__restrict__ err = A.err;
    const uint32_t a_slice = ct_a_slice_bytes(AR), b_slice = ct_b_slice_bytes(NP);
    const uint32_t a_region = ct_a_region_bytes(AR);
    const uint32_t stage = ct_stage_bytes(NP, AR);
    const uint32_t c_off = a_region + kCtSlices * b_slice;     // c_xc[32], c_j[32] of the stage
    const size_t ntri = (size_t)nbf * (nbf + 1) / 2;            // packed upper triangle per matrix
    // CTA partial: XC and J upper triangles, packed (element (mu, nu), mu <= nu, at
    // nu (nu + 1) / 2 + mu), double-float, in shared memory when spart (else in HBM / L2)
    float2 *s_part = reinterpret_cast<float2 *>(smem + (size_t)nst * stage);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __shared__ float s_colf[2 * kCtMaxNbf];     // column scales of the current chunk (epilogue)
    __shared__ int s_coloff[2 * kCtMaxNbf];     // packed-triangle offset of column n, row 0
    __shared__ int s_colnu[2 * kCtMaxNbf];      // basis function of column n

    // zero the operand stages once: rows >= AR of A and >= 2 nbf of B are never written
    {
        uint4 *z = reinterpret_cast<uint4 *>(smem);
        const int n16 = (int)((size_t)nst * stage / 16);
        for (int i = threadIdx.x; i < n16; i += kCtThreads) z[i] = make_uint4(0u, 0u, 0u, 0u);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    if (threadIdx.x == 0) {
        for (int s = 0; s < nst; ++s) {
            mbar_init(&sh->a_full[s], 1);
            mbar_init(&sh->full[s], kCtGroupWarps);      // the warps of the slot's group
            mbar_init(&sh->empty[s], 1);
        }
        mbar_init(&sh->tmem_full, 1);
        mbar_init(&sh->tmem_empty, 1);
        mbar_init(&sh->drain, 1);
        sh->fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    pdl_wait();      // the set-up above reads nothing the preceding kernels write

    if (warp < kCtProducers) {
        // ------------------------------------------------------------ producers
        // two groups of six warps own the even and the odd ring slots (nst is
        // even, so each group sees its slots' phases in order); in a group, warp
        // w takes row groups w, w + 6, ...; lane = (8-point group g) x (row within
        // the group of 8).  The eight lanes of one 16-byte shared-memory phase
        // share g and cover the eight rows of one core matrix, 128 contiguous
        // bytes, so the slice loads and stores are free of bank conflicts.
        const int grp = warp / kCtGroupWarps, wg = warp % kCtGroupWarps;
        const int g = lane >> 3, mrow = lane & 7;
        int it = 0;
        bool ok = true;
        for (int ch = (G ? vb_ : (int)blockIdx.x); ch < nchunk && ok; ch += (G ? nvb_ : (int)gridDim.x)) {
            const int kb0 = ch * kb_per_chunk, kb1 = min(nkb, kb0 + kb_per_chunk);
            const int2 ce = chunk_bounds(ch);
            const float sx = pow2f(-ce.x), sj = pow2f(-ce.y);
            // B row scales of this lane's rows for the chunk, in registers
            float rfr[kCtRowSteps];
            {
                const int *ea = rowexp + (size_t)ch * nbf, *es = swexp + (size_t)ch * nbf;
#pragma unroll
                for (int j = 0; j < kCtRowSteps; ++j) {
                    const int mu = 8 * kCtGroupWarps * j + 8 * wg + mrow;
                    rfr[j] = mu < nbf ? pow2f(max(-126, min(127, ea[mu] - es[mu]))) : 0.f;
                }
            }
            for (int kb = kb0; kb < kb1; ++kb, ++it) {
                const int s = it % nst, n = it / nst;
                if ((s & 1) != grp) continue;        // the other group's slot
                int w_ok = 1;
                if (lane == 0) w_ok = mbar_wait(&sh->a_full[s], (uint32_t)(n & 1)) ? 1 : 0;
                w_ok = __shfl_sync(0xffffffffu, w_ok, 0);
                if (!w_ok || sh->fail) {
                    if (lane == 0 && !w_ok) { atomicExch(err, 11); sh->fail = 1; }
                    ok = false;
                    break;
                }
                unsigned char *sA = smem + (size_t)s * stage;
                unsigned char *sB = sA + a_region;
                const float *sc = reinterpret_cast<const float *>(sA + c_off);
                float2 cx[4], cy[4];
#pragma unroll
                for (int k = 0; k < 4; ++k) {
                    cx[k] = f2mul(*reinterpret_cast<const float2 *>(sc + 8 * g + 2 * k), make_float2(sx, sx));
                    cy[k] = f2mul(*reinterpret_cast<const float2 *>(sc + kCtKS + 8 * g + 2 * k), make_float2(sj, sj));
                }
                // the lane's rows one at a time: its slice loads first, then the
                // arithmetic (predicated, no early exit)
#pragma unroll
                for (int j0 = 0; j0 < kCtRowSteps; j0 += 1) {
                    uint4 q0[1], q1[1], q2[1];
#pragma unroll
                    for (int jj = 0; jj < 1; ++jj) {
                        const int mu = 8 * kCtGroupWarps * (j0 + jj) + 8 * wg + mrow;
                        if (mu < nbf) {
                            const uint32_t oa = core_off(mu, 8 * g, kCtKcores);
                            q0[jj] = *reinterpret_cast<const uint4 *>(sA + oa);
                            q1[jj] = *reinterpret_cast<const uint4 *>(sA + a_slice + oa);
                            q2[jj] = *reinterpret_cast<const uint4 *>(sA + 2 * a_slice + oa);
                        }
                    }
#pragma unroll
                    for (int jj = 0; jj < 1; ++jj) {
                        const int mu = 8 * kCtGroupWarps * (j0 + jj) + 8 * wg + mrow;
                        if (mu < nbf) {
                            const uint32_t oa = core_off(mu, 8 * g, kCtKcores);
                            // B row scale: phi 2^(7 - e_mu) -> phi 2^(7 - s_mu)
                            const float2 rf = make_float2(rfr[j0 + jj], rfr[j0 + jj]);
                            float2 v[4], t[4];
                            unpack8(q0[jj], v);
                            unpack8(q1[jj], t);
#pragma unroll
                            for (int k = 0; k < 4; ++k) v[k] = f2add(v[k], t[k]);
                            unpack8(q2[jj], t);
                            float2 bx[4], by[4];
#pragma unroll
                            for (int k = 0; k < 4; ++k) {
                                v[k] = f2add(v[k], t[k]);              // phi 2^(7 - e_mu), |v| < 128
                                const float2 u = f2mul(v[k], rf);
                                bx[k] = f2mul(cx[k], u);               // c phi 2^(7 - s_mu - v), |bx| < 128
                                by[k] = f2mul(cy[k], u);
                            }
                            uint4 sbx[kCtSlices], sby[kCtSlices];
                            slice8_fixed(bx, sbx);
                            slice8_fixed(by, sby);
                            const uint32_t oj = core_off(nbf + mu, 8 * g, kCtKcores);
#pragma unroll
                            for (int i = 0; i < kCtSlices; ++i) {
                                *reinterpret_cast<uint4 *>(sB + i * b_slice + oa) = sbx[i];
                                *reinterpret_cast<uint4 *>(sB + i * b_slice + oj) = sby[i];
                            }
                        }
                    }
                }
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                __syncwarp();
                if (lane == 0) mbar_arrive(&sh->full[s]);
            }
        }
    } else if (warp == kCtMmaWarp) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(kCtM, NP);
            const uint32_t lbo = 128, sbo = kCtKcores * 128;
            // descriptors built once; every operand is a fixed byte offset from these
            const uint64_t desc0 = smem_desc(smem, lbo, sbo);
            const uint32_t d_hi = tmem, d_lo = tmem + 256;
            int it = 0, cc = 0;
            bool ok = true;
            for (int ch = (G ? vb_ : (int)blockIdx.x); ch < nchunk && ok; ch += (G ? nvb_ : (int)gridDim.x), ++cc) {
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
                    const uint64_t a_st = desc_add(desc0, (uint32_t)s * stage);
                    const uint64_t b_st = desc_add(a_st, a_region);
#pragma unroll
                    for (int kk = 0; kk < kCtKS / 16; ++kk) {
                        const uint32_t ko = (uint32_t)kk * 2 * lbo;
#pragma unroll
                        for (int i = 0; i < kCtSlices; ++i)
#pragma unroll
                            for (int j = 0; i + j < kCtSlices; ++j) {
                                const uint64_t ad = desc_add(a_st, i * a_slice + ko);
                                const uint64_t bd = desc_add(b_st, j * b_slice + ko);
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
    } else if (warp < kCtLoaderWarp) {
        // ------------------------------------------------------------ epilogue
        const int q = warp & 3;                  // TMEM lane quarter of this warp
        const int h = (warp - kCtEpi0) >> 2;     // column blocks h, h + kCtEpiWarps / 4, ...
        const int r = q * 32 + lane;             // accumulator row = basis function mu
        float2 *gpart = part + (size_t)(G ? vb_ : (int)blockIdx.x) * 2 * ntri;   // this CTA's partial in HBM
        int cc = 0;
        for (int ch = (G ? vb_ : (int)blockIdx.x); ch < nchunk; ch += (G ? nvb_ : (int)gridDim.x), ++cc) {
            const int kb0 = ch * kb_per_chunk, kb1 = min(nkb, kb0 + kb_per_chunk);
            // column scales 2^(s_nu + v - 14) of the chunk in shared memory, row scale 2^e_mu in a register
            {
                const int2 ce = chunk_bounds(ch);
                const int *es = swexp + (size_t)ch * nbf;
                for (int n = threadIdx.x - 32 * kCtEpi0; n < 2 * nbf; n += 32 * kCtEpiWarps) {
                    const int nu = n < nbf ? n : n - nbf;
                    const int e = es[nu] + (n < nbf ? ce.x : ce.y) - 14;
                    s_colf[n] = pow2f(max(-126, min(127, e)));
                    if (cc == 0) {
                        s_colnu[n] = nu;
                        s_coloff[n] = (n < nbf ? 0 : (int)ntri) + nu * (nu + 1) / 2;
                    }
                }
            }
            const float fr = r < nbf ? pow2f(max(-126, min(127, rowexp[(size_t)ch * nbf + r]))) : 0.f;
            const bool ok = mbar_wait(&sh->tmem_full, (uint32_t)(cc & 1));
            if (!ok) { atomicExch(err, 14); sh->fail = 1; }
            ct_epi_bar();
            if (sh->fail) break;
            tc_fence_after();
            const uint32_t ta = tmem + ((uint32_t)(q * 32) << 16);
            // the partial is either shared or global memory: one inlined copy of
            // the drain per space, so its accesses compile to the space's own
            // loads and stores instead of generic ones
            auto drain = [&](float2 *__restrict__ pxs) {
                for (int c0 = 16 * h; c0 < NP; c0 += 16 * (kCtEpiWarps / 4)) {
#pragma unroll
                    for (int hh = 0; hh < 16; hh += 8) {
                        // eight columns: D_hi and D_lo from TMEM, the column tables and
                        // old values, then the arithmetic, then the stores
                        float dh[8], dl[8];
                        tmem_ld8(ta + (uint32_t)(c0 + hh), dh);
                        tmem_ld8(ta + 256u + (uint32_t)(c0 + hh), dl);
                        tmem_wait_ld();
                        if (r < nbf) {
                            // (s, e) += (D_hi + D_lo) 2^(e_mu + s_nu + v - 14) for the
                            // upper-triangle elements
                            const int kend = min(8, 2 * nbf - c0 - hh);
                            int off[8];
                            float fk[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                const bool v = k < kend && r <= s_colnu[c0 + hh + k];
                                off[k] = v ? s_coloff[c0 + hh + k] + r : -1;
                                fk[k] = v ? s_colf[c0 + hh + k] * fr : 0.f;   // exact power of two
                            }
                            float2 old[8];
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                old[k] = (cc > 0 && off[k] >= 0) ? pxs[off[k]] : make_float2(0.f, 0.f);
#pragma unroll
                            for (int k = 0; k < 8; ++k) {
                                const float vh = dh[k] * fk[k], vl = dl[k] * fk[k];
                                float s2 = old[k].x, e2 = old[k].y;
                                const float t = s2 + vh;
                                const float bp = t - s2;
                                e2 += (s2 - (t - bp)) + (vh - bp) + vl;
                                s2 = t + e2;                             // renormalise: |e| <= ulp(s) / 2
                                old[k] = make_float2(s2, e2 - (s2 - t));
                            }
#pragma unroll
                            for (int k = 0; k < 8; ++k)
                                if (off[k] >= 0) pxs[off[k]] = old[k];
                        }
                    }
                }
            };
            if (spart) drain(s_part);
            else drain(gpart);
            tc_fence_before();
            ct_epi_bar();                        // all TMEM reads of this chunk are done
            if (threadIdx.x == 32 * kCtEpi0) mbar_arrive(&sh->tmem_empty);
        }
        if (spart && !sh->fail) {
            for (size_t i = threadIdx.x - 32 * kCtEpi0; i < 2 * ntri; i += 32 * kCtEpiWarps) gpart[i] = s_part[i];
        }
    } else {
        // ------------------------------------------------------------ loader
        if (lane == 0) {
            const uint32_t tx = kCtSlices * a_slice + 2 * kCtKS * 4;
            int it = 0, issued = 0;
            for (int ch = (G ? vb_ : (int)blockIdx.x); ch < nchunk; ch += (G ? nvb_ : (int)gridDim.x)) {
                const int kb0 = ch * kb_per_chunk, kb1 = min(nkb, kb0 + kb_per_chunk);
                bool ok = true;
                // L2 prefetch: this chunk's A block (first chunk only) and the next chunk's
                for (int pc = (ch == (G ? vb_ : (int)blockIdx.x) ? ch : ch + (G ? nvb_ : (int)gridDim.x)); pc <= ch + (G ? nvb_ : (int)gridDim.x); pc += (G ? nvb_ : (int)gridDim.x)) {
                    if (pc >= nchunk) break;
                    const int p0 = pc * kb_per_chunk, p1 = min(nkb, p0 + kb_per_chunk);
                    for (int kb = p0; kb < p1; ++kb)
                        prefetch_l2(aslices + (size_t)kb * kCtSlices * a_slice, kCtSlices * a_slice);
                }
                for (int kb = kb0; kb < kb1; ++kb, ++it) {
                    const int s = it % nst, n = it / nst;
                    if (!mbar_wait(&sh->empty[s], (uint32_t)((n & 1) ^ 1)) || sh->fail) {
                        atomicExch(err, 15);
                        sh->fail = 1;
                        ok = false;
                        break;
                    }
                    unsigned char *sA = smem + (size_t)s * stage;
                    mbar_arrive_expect_tx(&sh->a_full[s], tx);
                    bulk_g2s(sA, aslices + (size_t)kb * kCtSlices * a_slice, kCtSlices * a_slice, &sh->a_full[s]);
                    bulk_g2s(sA + c_off, cxc + (size_t)kb * kCtKS, kCtKS * 4, &sh->a_full[s]);
                    bulk_g2s(sA + c_off + kCtKS * 4, cj + (size_t)kb * kCtKS, kCtKS * 4, &sh->a_full[s]);
                    issued = it + 1;
                }
                if (!ok) break;
            }
            // drain: the copies of the last nst stages must land before the CTA exits
            for (int j = (issued > nst ? issued - nst : 0); j < issued; ++j)
                mbar_wait(&sh->a_full[j % nst], (uint32_t)((j / nst) & 1));
        }
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    const bool ok = sh->fail == 0;
    if (threadIdx.x == 0) {
        for (int s = 0; s < nst; ++s) {
            mbar_inval(&sh->a_full[s]);
            mbar_inval(&sh->full[s]);
            mbar_inval(&sh->empty[s]);
        }
        mbar_inval(&sh->tmem_full);
        mbar_inval(&sh->tmem_empty);
        mbar_inval(&sh->drain);
    }
    return ok;
}

__device__ __forceinline__ void contract_tc_alloc()
{
    CtShared *sh = &ct_sh;
    if ((threadIdx.x >> 5) == kCtMmaWarp) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(kCtTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// after the CTA's last __syncthreads
__device__ __forceinline__ void contract_tc_free(uint32_t tmem)
{
    if ((threadIdx.x >> 5) == kCtMmaWarp) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kCtTmemCols) : "memory");
    }
}

__global__ void __launch_bounds__(kCtThreads, 1) k_contract_tc(const CtArgs args)
{
    contract_tc_alloc();
    const uint32_t tmem = ct_sh.tmem_base;
    contract_tc_cta<false>(args, 0, 0, tmem);
    contract_tc_free(tmem);
    pdl_signal();
}

// the batch's grouped launch: items (molecule, virtual CTA) from the queue,
// TMEM allocated once for all of them
__global__ void __launch_bounds__(kCtThreads, 1) k_contract_tc_group(const CtArgs *__restrict__ args, GroupQueue q)
{
    contract_tc_alloc();
    const uint32_t tmem = ct_sh.tmem_base;
    gq_run(q, &ct_sh.item, [&](int m, int vb, int nvb) {
        const CtArgs a = args[m];
        return contract_tc_cta<true>(a, vb, nvb, tmem);
    });
    tc_fence_before();
    __syncthreads();
    contract_tc_free(tmem);
}

// ------------------------------------------------------------------ setup

// exponent bounds of max |phi_mu| and max |w phi_mu| over each chunk: block
// per chunk, warp per row
__global__ void k_ct_rowexp(int nbf, size_t npad, int nkb, int kb_per_chunk, const float *__restrict__ phi,
                            const double *__restrict__ W, int *__restrict__ rowexp, int *__restrict__ swexp)
{
    const int ch = blockIdx.x, warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const size_t p0 = (size_t)ch * kb_per_chunk * kCtKS;
    const size_t p1 = (size_t)min(nkb, (ch + 1) * kb_per_chunk) * kCtKS;
    for (int mu = warp; mu < nbf; mu += blockDim.x >> 5) {
        uint32_t m = 0u;
        double mw = 0.0;
        for (size_t p = p0 + lane; p < p1; p += 32) {
            const float f = phi[(size_t)mu * npad + p];
            m = max(m, __float_as_uint(f) & 0x7fffffffu);
            mw = fmax(mw, fabs(W[p] * (double)f));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
            mw = fmax(mw, __shfl_xor_sync(0xffffffffu, mw, o));
        }
        if (lane == 0) {
            rowexp[(size_t)ch * nbf + mu] = exp_bound(m);
            int e = 0;
            if (mw > 0.0) frexp(mw, &e);           // mw < 2^e
            swexp[(size_t)ch * nbf + mu] = e < kCtExpMin ? kCtExpMin : (e > kCtExpMax ? kCtExpMax : e);
        }
    }
}

// 1 / w in FP32 (0 where the weight vanishes), for the per-build bound of |c / w|
__global__ void k_ct_winv(size_t npad, const double *__restrict__ W, float *__restrict__ winv)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p < npad) winv[p] = W[p] > 1e-30 ? (float)(1.0 / W[p]) : 0.f;
}

// A slices in HBM, [nkb][slice][AR x 32 core layout]: thread per (kb, row, 8-point group)
// the three BF16 slices of the FP32 amplitudes (the ones the B operand and the
// CUDA-core path use), in FP32 arithmetic: x = phi 2^(7 - e) and every remainder
// are exact in FP32, so the slices are those of the exact values
__global__ void k_ct_slice_A(int nbf, int AR, size_t npad, int nkb, int kb_per_chunk, const float *__restrict__ phi,
                             const int *__restrict__ rowexp, __nv_bfloat16 *__restrict__ A)
{
    const size_t id = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t total = (size_t)nkb * AR * 4;
    if (id >= total) return;
    const int g = (int)(id & 3);
    const int row = (int)((id >> 2) % AR);
    const int kb = (int)(id / ((size_t)AR * 4));
    const size_t blk = (size_t)AR * kCtKS;                  // elements of one slice block
    const uint32_t o = core_off(row, 8 * g, kCtKcores) / 2;
    const int e = row < nbf ? rowexp[(size_t)(kb / kb_per_chunk) * nbf + row] : 0;
    for (int k = 0; k < 8; ++k) {
        const size_t p = (size_t)kb * kCtKS + 8 * g + k;
        const float x = row < nbf ? phi[(size_t)row * npad + p] * pow2f(7 - e) : 0.f;   // |7 - e| <= 107
        const float a1 = rintf(x);
        const float r1 = x - a1;
        const __nv_bfloat16 h2 = __float2bfloat16_rn(r1);
        const float r2 = r1 - __bfloat162float(h2);
        const size_t base = (size_t)kb * kCtSlices * blk + o + k;
        A[base] = __float2bfloat16_rn(a1);
        A[base + blk] = h2;
        A[base + 2 * blk] = __float2bfloat16_rn(r2);
    }
}

static size_t ct_smem(int nst, int NP, int AR, int nbf, bool spart)
{
    return (size_t)nst * ct_stage_bytes(NP, AR) + (spart ? (size_t)nbf * (nbf + 1) * sizeof(float2) : 0);
}

__device__ __forceinline__ void contract_tc_reduce_block(const RedArgs A, int vb)
{
    __shared__ float2 shx[32][33], shj[32][33];
    const int nbf = A.nbf, nparts = A.nparts;
    const float2 *__restrict__ part = A.part;
    const size_t nn = (size_t)nbf * nbf, ntri = (size_t)nbf * (nbf + 1) / 2;
    const int lx = threadIdx.x & 31, g = threadIdx.x >> 5;
    const size_t e = (size_t)vb * 32 + lx;                  // element (mu, nu) = e % nbf, e / nbf
    const int nu = (int)(e / nbf), mu = (int)(e % nbf);
    const bool act = e < nn && mu <= nu;
    const size_t t = (size_t)nu * (nu + 1) / 2 + mu;        // packed upper-triangle index
    if (vb == 0 && A.sc && threadIdx.x < 3)                  // the build's E_xc, N, E_J
        A.sc[threadIdx.x] = A.scal[threadIdx.x == 0 ? kScalExc : (threadIdx.x == 1 ? kScalNelec : kScalEJ)];
    if (vb == 0 && A.cmax)                                   // chunk maxima start from zero next build
        for (int i = threadIdx.x; i < A.ncmax; i += blockDim.x) A.cmax[i] = 0u;
    dfl sx{0.f, 0.f}, sj{0.f, 0.f};
    if (act)
        for (int c = g; c < nparts; c += 32) {
            const float2 *p = part + (size_t)c * 2 * ntri;
            const float2 a = p[t], b = p[ntri + t];
            sx = df_add(sx, dfl{a.x, a.y});
            sj = df_add(sj, dfl{b.x, b.y});
        }
    shx[g][lx] = make_float2(sx.h, sx.l);
    shj[g][lx] = make_float2(sj.h, sj.l);
    __syncthreads();
    if (g != 0 || !act) return;
    for (int k = 1; k < 32; ++k) {
        sx = df_add(sx, dfl{shx[k][lx].x, shx[k][lx].y});
        sj = df_add(sj, dfl{shj[k][lx].x, shj[k][lx].y});
    }
    const double vx = df_to(sx), vj = df_to(sj);
    const size_t lo = (size_t)nu * nbf + mu, up = (size_t)mu * nbf + nu;
    if (A.want_xc) {
        A.XC[lo] = vx;
        A.XC[up] = vx;
        if (A.XC2) {
            A.XC2[lo] = vx;
            A.XC2[up] = vx;
        }
    }
    if (A.want_j) {
        A.J[lo] = vj;
        A.J[up] = vj;
        if (A.J2) {
            A.J2[lo] = vj;
            A.J2[up] = vj;
        }
    }
}

// Sum the double-float CTA partials of every element on or above the diagonal
// in CTA order (double-float, no FP64 until the final value) and write XC, J
// symmetrically (column-major).  Block: 32 elements x 32 CTA groups; group g
// sums CTAs g, g + 32, ...; the 32 group sums are added in a fixed order.
__global__ void __launch_bounds__(1024) k_contract_tc_reduce(const RedArgs a)
{
    pdl_wait();
    contract_tc_reduce_block(a, (int)blockIdx.x);
    pdl_signal();
}

__global__ void __launch_bounds__(1024) k_contract_tc_reduce_group(const RedArgs *__restrict__ args, GroupQueue q)
{
    __shared__ int s_item;
    gq_run(q, &s_item, [&](int m, int vb, int) {
        const RedArgs a = args[m];
        contract_tc_reduce_block(a, vb);
        return true;
    });
}

// chunking of the point dimension for nsm CTAs: chunks per CTA is the smallest
// count that keeps every chunk at most kCtMaxKbPerChunk stages long
static void ct_plan(size_t npad, int nsm, int &nkb, int &kbpc, int &nchunk)
{
    nkb = (int)(npad / kCtKS);
    const int per_cta = (nkb + nsm * kCtMaxKbPerChunk - 1) / (nsm * kCtMaxKbPerChunk);
    const int target = nsm * (per_cta > 0 ? per_cta : 1);
    kbpc = (nkb + target - 1) / target;
    if (kbpc < 1) kbpc = 1;
    nchunk = (nkb + kbpc - 1) / kbpc;
}

size_t contract_tc_part_elems(int nbf, size_t npad, int nsm)
{
    if (nbf > kCtMaxNbf) return 0;
    int nkb, kbpc, nchunk;
    ct_plan(npad, nsm, nkb, kbpc, nchunk);
    const int grid = nchunk < nsm ? nchunk : nsm;
    return (size_t)grid * nbf * (nbf + 1);        // one packed partial (XC and J triangles) per CTA
}

int contract_tc_setup(dftg_ctx *c)
{
    if (c->nbf > kCtMaxNbf) return DFTG_OK;
    int nsm = 0, optin = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    DFTG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
    const int NP = (2 * c->nbf + 15) / 16 * 16;
    const int AR = (c->nbf + 7) / 8 * 8;
    cudaFuncAttributes fa{};
    DFTG_CUDA(cudaFuncGetAttributes(&fa, k_contract_tc));
    optin -= (int)fa.sharedSizeBytes;                 // static shared memory of the kernel
    // keep the CTA partial in shared memory if at least three stages still fit
    bool spart = true;
    int nst = kCtMaxStages;
    while (nst > 3 && ct_smem(nst, NP, AR, c->nbf, spart) > (size_t)optin) --nst;
    if (ct_smem(nst, NP, AR, c->nbf, spart) > (size_t)optin) {
        spart = false;
        nst = kCtMaxStages;
        while (nst > 2 && ct_smem(nst, NP, AR, c->nbf, spart) > (size_t)optin) --nst;
    }
    nst &= ~1;                                        // the producer groups own even / odd slots
    if (nst < 2 || ct_smem(nst, NP, AR, c->nbf, spart) > (size_t)optin) return DFTG_OK;
    int nkb, kbpc, nchunk;
    ct_plan(c->npad, nsm, nkb, kbpc, nchunk);
    const int grid = nchunk < nsm ? nchunk : nsm;
    if ((size_t)grid * c->nbf * (c->nbf + 1) > c->part_elems) return DFTG_OK;
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_contract_tc), c->device));
    if (!c->d_flag) {
        DFTG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
    }
    DFTG_CUDA(cudaMalloc(&c->d_ct_rowexp, sizeof(int) * 2 * (size_t)nchunk * c->nbf + sizeof(int2) * (size_t)nchunk));
    DFTG_CUDA(cudaMalloc(&c->d_ct_winv, sizeof(float) * c->npad));
    DFTG_CUDA(cudaMalloc(&c->d_ct_A, sizeof(__nv_bfloat16) * (size_t)nkb * kCtSlices * AR * kCtKS));
    k_ct_rowexp<<<nchunk, 256, 0, c->stream>>>(c->nbf, c->npad, nkb, kbpc, c->d_phi32, c->d_w, c->d_ct_rowexp,
                                               c->d_ct_rowexp + (size_t)nchunk * c->nbf);
    DFTG_LAUNCH_CHECK();
    k_ct_winv<<<(unsigned)((c->npad + 255) / 256), 256, 0, c->stream>>>(c->npad, c->d_w, c->d_ct_winv);
    DFTG_LAUNCH_CHECK();
    const size_t threads = (size_t)nkb * AR * 4;
    k_ct_slice_A<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->nbf, AR, c->npad, nkb, kbpc, c->d_phi32, c->d_ct_rowexp, reinterpret_cast<__nv_bfloat16 *>(c->d_ct_A));
    DFTG_LAUNCH_CHECK();
    DFTG_CUDA(cudaMalloc(&c->d_ct_cmax, sizeof(unsigned) * 2 * (size_t)nchunk));
    DFTG_CUDA(cudaMemsetAsync(c->d_ct_cmax, 0, sizeof(unsigned) * 2 * (size_t)nchunk, c->stream));
    c->ct_NP = NP;
    c->ct_AR = AR;
    c->ct_nst = nst;
    c->ct_spart = spart ? 1 : 0;
    c->ct_nkb = nkb;
    c->ct_kbpc = kbpc;
    c->ct_nchunk = nchunk;
    c->ct_grid = grid;
    c->ct_grid_max = grid;
    c->ct_nst_max = nst;
    // fewest stages the autotuner may choose: a CTA still needs more than half
    // of the shared memory, so one contraction CTA runs per SM as at setup
    int nmin = nst;
    while (nmin > 2 && ct_smem(nmin - 1, NP, AR, c->nbf, spart) * 2 > (size_t)optin) --nmin;
    nmin = (nmin + 1) & ~1;                           // even ring depths only
    c->ct_nst_min = nmin < nst ? nmin : nst;
    c->ct_ready = true;
    return DFTG_OK;
}

StepLaunch<CexpArgs> step_cexp(const dftg_ctx *c, const float *cx, const float *cy)
{
    StepLaunch<CexpArgs> s;
    s.args = CexpArgs{c->ct_nkb, c->ct_kbpc, cx, cy, c->d_ct_winv,
                      reinterpret_cast<int2 *>(c->d_ct_rowexp + 2 * (size_t)c->ct_nchunk * c->nbf)};
    s.blocks = c->ct_nchunk;
    return s;
}

StepLaunch<CtArgs> step_contract_tc(const dftg_ctx *c, const float *cx, const float *cy)
{
    StepLaunch<CtArgs> s;
    s.args = CtArgs{c->nbf, c->ct_AR, c->ct_NP, c->ct_nst, c->ct_spart, c->ct_nkb, c->ct_kbpc, c->ct_nchunk,
                    reinterpret_cast<const unsigned char *>(c->d_ct_A), c->d_ct_rowexp,
                    c->d_ct_rowexp + (size_t)c->ct_nchunk * c->nbf,
                    reinterpret_cast<const int2 *>(c->d_ct_rowexp + 2 * (size_t)c->ct_nchunk * c->nbf), cx, cy,
                    reinterpret_cast<float2 *>(c->d_part), c->d_flag,
                    cmax_route(c) && cx == c->d_cxc32 && cy == c->d_cj32 ? c->d_ct_cmax : nullptr};
    s.blocks = c->ct_grid;
    s.smem = ct_smem(c->ct_nst, c->ct_NP, c->ct_AR, c->nbf, c->ct_spart != 0);
    return s;
}

StepLaunch<RedArgs> step_contract_reduce(const dftg_ctx *c, bool want_xc, bool want_j, double *XC, double *J)
{
    StepLaunch<RedArgs> s;
    s.args = RedArgs{c->nbf, c->ct_grid, want_xc ? 1 : 0, want_j ? 1 : 0, reinterpret_cast<const float2 *>(c->d_part),
                     XC, J, nullptr, nullptr, c->d_scal, nullptr, cmax_route(c) ? c->d_ct_cmax : nullptr,
                     2 * c->ct_nchunk};
    s.blocks = (int)(((size_t)c->nbf * c->nbf + 31) / 32);
    return s;
}

// XC = phi^T diag(cxc) phi and J = phi^T diag(cj) phi partials on the tensor
// cores for any pair of FP32 point-coefficient arrays
int launch_contract_tc_on(dftg_ctx *c, const float *cxc32, const float *cj32)
{
    const StepLaunch<CtArgs> ct = step_contract_tc(c, cxc32, cj32);
    if (!ct.args.cmax) {                 // the bounds pass (the whole build keeps chunk maxima instead)
        const StepLaunch<CexpArgs> ce = step_cexp(c, cxc32, cj32);
        k_ct_cexp<<<ce.blocks, kCexpThreads, 0, c->stream>>>(ce.args);
        DFTG_LAUNCH_CHECK();
        DFTG_MARK(c, "contract_bounds");
    }
    DFTG_CUDA(launch_pdl(k_contract_tc, ct.blocks, kCtThreads, ct.smem, c->stream, ct.args));
    return DFTG_OK;
}

int launch_contract_tc(dftg_ctx *c) { return launch_contract_tc_on(c, c->d_cxc32, c->d_cj32); }

// Set-up tables shared with the tiled kernel for nbf > 128 (k_contract_tt.cu):
// per-chunk exponent bounds of |phi| and |w phi|, 1 / w, and the BF16 slices of
// phi in the [nkb][3][AR x 32] operand layout (rows nbf .. AR - 1 zero)
int ct_setup_tables(dftg_ctx *c, int AR, int nkb, int kbpc, int nchunk, int *rowexp, int *swexp, float *winv,
                    void *A)
{
    k_ct_rowexp<<<nchunk, 256, 0, c->stream>>>(c->nbf, c->npad, nkb, kbpc, c->d_phi32, c->d_w, rowexp, swexp);
    DFTG_LAUNCH_CHECK();
    k_ct_winv<<<(unsigned)((c->npad + 255) / 256), 256, 0, c->stream>>>(c->npad, c->d_w, winv);
    DFTG_LAUNCH_CHECK();
    const size_t threads = (size_t)nkb * AR * 4;
    k_ct_slice_A<<<(unsigned)((threads + 255) / 256), 256, 0, c->stream>>>(
        c->nbf, AR, c->npad, nkb, kbpc, c->d_phi32, rowexp, reinterpret_cast<__nv_bfloat16 *>(A));
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// per-chunk exponent bounds of |c_x / w| and |c_y / w| (one build)
int ct_launch_cexp(dftg_ctx *c, int nkb, int kbpc, int nchunk, const float *cx, const float *cy, const float *winv,
                   int2 *cexp)
{
    k_ct_cexp<<<nchunk, kCexpThreads, 0, c->stream>>>(CexpArgs{nkb, kbpc, cx, cy, winv, cexp});
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int launch_contract_tc_reduce_to(dftg_ctx *c, bool want_xc, bool want_j, double *XC, double *J)
{
    const StepLaunch<RedArgs> st = step_contract_reduce(c, want_xc, want_j, XC, J);
    DFTG_CUDA(launch_pdl(k_contract_tc_reduce, st.blocks, 1024, 0, c->stream, st.args));
    return DFTG_OK;
}

int group_cexp(const CexpArgs *d_args, const GroupQueue &q, int nsm, cudaStream_t st)
{
    int occ = 0;
    DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_ct_cexp_group, kCexpThreads, 0));
    const int grid = group_grid(q, occ, nsm);
    if (grid > 0) k_ct_cexp_group<<<grid, kCexpThreads, 0, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int group_contract_tc(const CtArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st)
{
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_contract_tc_group), device));
    // one CTA per SM: each holds all kCtTmemCols TMEM columns for its lifetime
    const int grid = group_grid(q, 1, nsm);
    if (grid > 0) k_contract_tc_group<<<grid, kCtThreads, smem, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int group_contract_reduce(const RedArgs *d_args, const GroupQueue &q, int nsm, cudaStream_t st)
{
    int occ = 0;
    DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_contract_tc_reduce_group, 1024, 0));
    const int grid = group_grid(q, occ, nsm);
    if (grid > 0) k_contract_tc_reduce_group<<<grid, 1024, 0, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int launch_contract_tc_reduce(dftg_ctx *c, bool want_xc, bool want_j)
{
    return launch_contract_tc_reduce_to(c, want_xc, want_j, c->d_XC, c->d_J);
}

}  // namespace dftg
