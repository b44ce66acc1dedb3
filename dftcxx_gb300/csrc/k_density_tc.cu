// k_density_tc.cu -- mixed-path density rho_p = 2 phi_p^T P phi_p on the tcgen05
// tensor cores, accurate to ~1e-8 relative (gridpoint.cpp:82-84).
//
// The energy depends on rho at first order, so rho must carry near-FP64
// accuracy; FP32 or 3xTF32 arithmetic leaves ~1e-7 random errors per point,
// about 3e-6 Ha on benzene.  The GEMM T = Phi P is therefore done as an
// integer-slice product (Ozaki's error-free splitting) on the FP16 tensor cores,
// with three fixed-point slices per operand:
//
//   Phi[p, mu] 2^(8 - e_p) = A_1 + A_2 + 2^-11 A_3      (per point e_p, |Phi| < 2^e_p)
//   P[mu, nu]  2^(8 - t_nu) = B_1 + B_2 + 2^-11 B_3     (per column t_nu)
//
// A_1 an integer (|A_1| <= 256), A_2 and A_3 multiples of 2^-11 (|.| <= 1/2):
// balanced base-2^11 digits of the operand rounded to 2^-30 of 2^e, every
// slice exact in FP16 (formed with integer operations on the IEEE bits).  Three accumulators per tile:
//   D_hi  = A_1 B_1                               integer products, exact in FP32
//   D_lo  = A_1 B_2 + A_2 B_1 + A_2 B_2            about 2^-9 of D_hi
//   D_lo2 = A_1 B_3 + A_3 B_1 + A_2 B_3 + A_3 B_2  weight 2^-11
// (A_3 B_3, 2^-22 x 2^-22 of the head, is dropped): eight MMAs per K step.  The
// epilogue forms T = D_hi + D_lo + 2^-11 D_lo2 with TwoSum and rho = 2 sum_nu
// T_nu phi_nu in compensated FP32, phi rebuilt exactly from the slices in
// shared memory (A_1 + A_2 is exact in FP32).  Six bytes per operand element.
//
// Layouts (canonical no-swizzle K-major core matrices, 8 rows x 16 bytes,
// cores ordered row group by row group: LBO 128 B, SBO (KP/8) 128 B):
//   A slices in HBM: [slice][tile][128/8][KP/8][8][8] FP16, one contiguous
//     128 x KP block per slice and tile, copied with cp.async.bulk;
//   B slices: [slice][NP/8][KP/8][8][8] FP16 (rows nu, K = mu).
// CTA: warp 0 producer (bulk copies), warp 1 TMEM owner + MMA issuer,
// warps 2-17 epilogue in two groups of eight that take alternate tiles (group g
// the tiles of TMEM accumulator set g); TMEM lanes 32 (w % 4) ..., the two warps
// of a lane quarter in a group take alternate 8-column groups and meet in shared
// memory per tile.
// Whole-build form: the density correction's total is known before this pass,
// sum_p w rho = 2 tr(P S_grid) with S_grid = Phi^T diag(w) Phi made once per
// grid: the P-slicing step forms the column partials of the trace, the epilogue
// warps sum them (in a fixed order, before their first tile) into the factor,
// apply it, and write the rho w_becke planes for the
// multipoles (no atom-sum pass; the LDA point kernel then runs beside the
// Hartree steps).
// Persistent over tiles: three A stages and two TMEM accumulator sets, so the
// copies of the next tiles and the MMAs of one tile overlap the epilogue of the
// previous one.  Every mbarrier wait is bounded: on expiry the CTA records an
// error code, drains its copies, frees TMEM and exits.
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>
#include "dftg_internal.cuh"
#include "tc_common.cuh"

namespace dftg {

constexpr int kTcSlices = 3;
constexpr int kTcStages = 3;                  // A stages (copies in flight + the tile in use)
constexpr int kTcAcc = 80;                    // TMEM column stride of the three accumulators of a set
constexpr int kTcTile = 128;
constexpr int kTcMaxK = 80;                   // nbf <= 80 for this kernel
constexpr int kTcEpiWarps = 16;               // four per TMEM lane quarter
constexpr int kTcThreads = (2 + kTcEpiWarps) * 32;
constexpr uint32_t kTcTmemCols = 512;
// named barriers 1 and 2 over the eight warps of epilogue group 0 and 1
__device__ __forceinline__ void epi_group_bar(int g)
{
    asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "n"(kTcEpiWarps * 16) : "memory");
}

__device__ __forceinline__ void unpack8_f16(uint4 u, float (&v)[8])
{
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w[j]));
        v[2 * j] = f.x;
        v[2 * j + 1] = f.y;
    }
}

struct TcShared {
    uint64_t full[kTcStages], empty[kTcStages], tmem_full[2], tmem_empty[2];
    uint32_t tmem_base;
    int item;                              // the grouped launch's queue position (broadcast)
};

// the CTA's mbarriers and TMEM address (one instance in every kernel that uses them)
__shared__ TcShared tc_sh;

// The density correction factor sum Z / sum_p w rho with sum_p w rho =
// 2 tr(P S_grid) (moleculargrid.cpp:132-146), from the P-slicing step's column
// partials summed in a fixed order by the first epilogue warp (lanes over
// columns, then a fixed shuffle tree), so every CTA forms the same value;
// block 0 writes the total and the factor to scal.  Named barrier 3 over the
// epilogue warps.
__device__ __forceinline__ double density_factor(const DensTcArgs &a, int vb)
{
    __shared__ double s_cf;
    const int et = (int)threadIdx.x - 64, lane = threadIdx.x & 31;   // epilogue thread 0 .. 32 kTcEpiWarps - 1
    if (et < 32) {
        double t = 0.0, charge = 0.0;
        for (int n = lane; n < a.nbf; n += 32) t += a.tr[n];
        for (int i = lane; i < a.natoms; i += 32) charge += a.atoms[4 * i + 3];
        for (int o = 16; o > 0; o >>= 1) {
            t += __shfl_xor_sync(0xffffffffu, t, o);
            charge += __shfl_xor_sync(0xffffffffu, charge, o);
        }
        if (et == 0) {
            const double total = 2.0 * t;
            s_cf = charge / total;
            if (vb == 0) {
                a.scal[kScalSum] = total;
                a.scal[kScalScale] = s_cf;
            }
        }
    }
    asm volatile("bar.sync 3, %0;" ::"n"(kTcEpiWarps * 32) : "memory");
    return s_cf;
}

// One CTA's share of one molecule's tiles (vb, vb + nvb, ...): initialises the
// mbarriers, stages the B slices, runs the producer / MMA / epilogue roles and
// invalidates the mbarriers again.  The caller owns the kTcTmemCols TMEM
// columns at tmem.  Returns false (block-uniform) when a bounded wait gave up.

__device__ __forceinline__ bool density_tc_cta(const DensTcArgs args, int vb, int nvb, uint32_t tmem)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    TcShared *sh = &tc_sh;
    const int nbf = args.nbf, KP = args.KP, NP = args.NP, ntiles = args.ntiles;
    const unsigned char *__restrict__ Aslices = args.A;
    const int *__restrict__ row_exp = args.row_exp;
    const unsigned char *__restrict__ Bslices = args.B;
    const int *__restrict__ col_exp = args.col_exp;
    double *__restrict__ rho = args.rho;
    int *__restrict__ err = args.err;
    const uint32_t a_slice_bytes = (uint32_t)kTcTile * KP * 2;
    const uint32_t a_stage_bytes = kTcSlices * a_slice_bytes;
    const uint32_t b_slice_bytes = (uint32_t)NP * KP * 2;
    unsigned char *sA = smem;                                   // [stages][slices][tile block]
    unsigned char *sB = smem + kTcStages * a_stage_bytes;        // [slices][B block]
    __shared__ __align__(16) int s_texp[kTcMaxK];
    __shared__ int s_fail;
    __shared__ float2 s_part[2][kTcTile];         // (S, E) of the second column half of each epilogue group

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) {
        for (int b = 0; b < kTcStages; ++b) {
            mbar_init(&sh->full[b], 1);
            mbar_init(&sh->empty[b], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sh->tmem_full[b], 1);
            mbar_init(&sh->tmem_empty[b], 1);
        }
        s_fail = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // B slices and column exponents: plain copies, then made visible to the tensor core
    {
        const uint4 *src = reinterpret_cast<const uint4 *>(Bslices);
        uint4 *dst = reinterpret_cast<uint4 *>(sB);
        const int n16 = (int)(kTcSlices * b_slice_bytes / 16);
        for (int i = threadIdx.x; i < n16; i += kTcThreads) dst[i] = src[i];
        for (int i = threadIdx.x; i < NP && i < kTcMaxK; i += kTcThreads) s_texp[i] = i < nbf ? col_exp[i] : 0;
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const int my_tiles = (ntiles - vb + nvb - 1) / nvb;

    if (warp == 0) {
        // ------------------------------------------------------------ producer
        int issued = 0;
        if (lane == 0) {
            // L2 prefetch a ring's depth ahead of the bulk copies
            for (int it = 0; it < kTcStages && it < my_tiles; ++it)
                for (int i = 0; i < kTcSlices; ++i)
                    prefetch_l2(Aslices + ((size_t)i * ntiles + vb + it * nvb) * a_slice_bytes, a_slice_bytes);
            for (int it = 0; it < my_tiles; ++it) {
                const int s = it % kTcStages, n = it / kTcStages;
                if (it + kTcStages < my_tiles)
                    for (int i = 0; i < kTcSlices; ++i)
                        prefetch_l2(Aslices + ((size_t)i * ntiles + vb + (it + kTcStages) * nvb) * a_slice_bytes,
                                    a_slice_bytes);
                if (!mbar_wait(&sh->empty[s], (uint32_t)((n & 1) ^ 1))) { atomicExch(err, 1); s_fail = 1; break; }
                if (s_fail) break;
                const int tile = vb + it * nvb;
                mbar_arrive_expect_tx(&sh->full[s], a_stage_bytes);
                for (int i = 0; i < kTcSlices; ++i)
                    bulk_g2s(sA + (size_t)s * a_stage_bytes + (size_t)i * a_slice_bytes,
                             Aslices + ((size_t)i * ntiles + tile) * a_slice_bytes, a_slice_bytes, &sh->full[s]);
                issued = it + 1;
            }
            // drain: every issued stage must have landed before the CTA exits
            for (int it = (issued > kTcStages ? issued - kTcStages : 0); it < issued; ++it)
                mbar_wait(&sh->full[it % kTcStages], (uint32_t)((it / kTcStages) & 1));
        }
        __syncwarp();
    } else if (warp == 1) {
        // ------------------------------------------------------------ MMA issuer
        if (lane == 0) {
            const uint32_t idesc = idesc_f16(kTcTile, NP);
            const uint32_t lbo = 128, sbo = (uint32_t)(KP / 8) * 128;
            // descriptors built once; every operand is a fixed byte offset from these
            const uint64_t a_desc0 = smem_desc(sA, lbo, sbo), b_desc0 = smem_desc(sB, lbo, sbo);
            const int ksteps = KP / 16;
            for (int it = 0; it < my_tiles; ++it) {
                const int s = it % kTcStages, ns = it / kTcStages;   // A stage
                const int bset = it & 1, nb = it >> 1;               // TMEM accumulator set
                if (!mbar_wait(&sh->full[s], (uint32_t)(ns & 1))) { atomicExch(err, 2); s_fail = 1; break; }
                if (!mbar_wait(&sh->tmem_empty[bset], (uint32_t)((nb & 1) ^ 1))) { atomicExch(err, 3); s_fail = 1; break; }
                if (s_fail) break;
                tc_fence_after();
                const uint64_t a_st = desc_add(a_desc0, (uint32_t)s * a_stage_bytes);
                const uint32_t d_hi = tmem + (uint32_t)(bset * 256), d_lo = d_hi + kTcAcc, d_lo2 = d_hi + 2 * kTcAcc;
                // K step outermost (the tensor core reuses the K block's operands)
                for (int kk = 0; kk < ksteps; ++kk) {
                    const uint64_t ak = desc_add(a_st, kk * 2 * lbo), bk = desc_add(b_desc0, kk * 2 * lbo);
                    const uint64_t a1 = ak, a2 = desc_add(ak, a_slice_bytes), a3 = desc_add(ak, 2 * a_slice_bytes);
                    const uint64_t b1 = bk, b2 = desc_add(bk, b_slice_bytes), b3 = desc_add(bk, 2 * b_slice_bytes);
                    const uint32_t acc = kk > 0 ? 1u : 0u;
                    mma_bf16(d_hi, a1, b1, idesc, acc);
                    mma_bf16(d_lo, a1, b2, idesc, acc);
                    mma_bf16(d_lo, a2, b1, idesc, 1u);
                    mma_bf16(d_lo, a2, b2, idesc, 1u);
                    mma_bf16(d_lo2, a1, b3, idesc, acc);
                    mma_bf16(d_lo2, a3, b1, idesc, 1u);
                    mma_bf16(d_lo2, a2, b3, idesc, 1u);
                    mma_bf16(d_lo2, a3, b2, idesc, 1u);
                }
                mma_commit(&sh->tmem_full[bset]);
            }
        }
        __syncwarp();
    } else {
        // ------------------------------------------------------------ epilogue
        // two groups of eight warps take alternate tiles (group g the tiles of
        // TMEM accumulator set g), so two tiles' epilogues are in flight; in a
        // group, the two warps of a lane quarter take alternate 8-column groups
        const int q = warp & 3;                 // TMEM lane quarter of this warp
        const int eg = (warp - 2) >> 3;         // epilogue group = accumulator set
        const int half = ((warp - 2) >> 2) & 1; // 8-column groups 8 half, 8 half + 16, ...
        const int r = q * 32 + lane;            // row of the tile = TMEM lane
        const int kc = KP / 8;
        const double cf = args.correct ? density_factor(args, vb) : 1.0;
        for (int it = eg; it < my_tiles; it += 2) {
            const int s = it % kTcStages;
            const int nb = it >> 1;
            const int tile = vb + it * nvb;
            const size_t p = (size_t)tile * kTcTile + r;
            // the point's exponent and w_becke planes, loaded now and used at the
            // tile's end (their latency hidden behind the column loop)
            int ep = 0;
            float wbh = 0.f, wbl = 0.f;
            if (half == 0) {
                ep = row_exp[p];
                if (args.rw32) {
                    wbh = args.wb2[p];
                    wbl = args.wb2[args.npad + p];
                }
            }
            bool ok = mbar_wait(&sh->tmem_full[eg], (uint32_t)(nb & 1));
            if (!ok) { atomicExch(err, 4); s_fail = 1; }
            epi_group_bar(eg);
            if (s_fail) break;
            tc_fence_after();
            const unsigned char *a0 = sA + (size_t)s * a_stage_bytes;
            const uint32_t ta0 = tmem + (uint32_t)(eg * 256) + ((uint32_t)(q * 32) << 16);
            // two independent compensated accumulators (even / odd columns), the
            // two lanes of packed FP32 pairs: every step below is one packed
            // instruction for an (even, odd) column pair
            float2 S = make_float2(0.f, 0.f), E = make_float2(0.f, 0.f);
            const float2 k2m11 = make_float2(0x1p-11f, 0x1p-11f);
            // columns nu >= nbf hold T = 0 and phi = 0 (zero rows of B, zero slices
            // of A) and contribute exactly nothing, so every group is done whole
            for (int nb8 = 8 * half; nb8 < nbf; nb8 += 16) {
                float dh[8], dl[8], dl2[8];
                tmem_ld8(ta0 + (uint32_t)nb8, dh);
                tmem_ld8(ta0 + (uint32_t)(kTcAcc + nb8), dl);
                tmem_ld8(ta0 + (uint32_t)(2 * kTcAcc + nb8), dl2);
                // phi 2^(8 - e_p) of columns nb8..nb8+7 from the three slices (16 B each)
                const uint32_t off = core_off(r, nb8, kc);
                float m1[8], m2[8], m3[8];
                unpack8_f16(*reinterpret_cast<const uint4 *>(a0 + off), m1);
                unpack8_f16(*reinterpret_cast<const uint4 *>(a0 + a_slice_bytes + off), m2);
                unpack8_f16(*reinterpret_cast<const uint4 *>(a0 + 2 * a_slice_bytes + off), m3);
                const int4 e0 = *reinterpret_cast<const int4 *>(s_texp + nb8);
                const int4 e1 = *reinterpret_cast<const int4 *>(s_texp + nb8 + 4);
                const int ex[8] = {e0.x, e0.y, e0.z, e0.w, e1.x, e1.y, e1.z, e1.w};
                tmem_wait_ld();
#pragma unroll
                for (int k = 0; k < 8; k += 2) {
                    // T~_nu 2^16 = D_hi + D_lo + 2^-11 D_lo2 as u + te (TwoSum of the
                    // first two), scaled by 2^(t_nu - 24); phi~ 2^8 = fh + fl
                    const float2 h = make_float2(dh[k], dh[k + 1]), l = make_float2(dl[k], dl[k + 1]);
                    const float2 u = f2add(h, l);
                    const float2 bp = f2sub(u, h);
                    float2 te = f2fma(make_float2(dl2[k], dl2[k + 1]), k2m11,
                                      f2add(f2sub(h, f2sub(u, bp)), f2sub(l, bp)));
                    const float2 sc = make_float2(__int_as_float((127 - 24 + ex[k]) << 23),
                                                  __int_as_float((127 - 24 + ex[k + 1]) << 23));
                    const float2 t = f2mul(u, sc);
                    te = f2mul(te, sc);
                    // exact: multiples of 2^-11 below 2^9
                    const float2 fh = f2add(make_float2(m1[k], m1[k + 1]), make_float2(m2[k], m2[k + 1]));
                    const float2 fl = f2mul(make_float2(m3[k], m3[k + 1]), k2m11);
                    // S + E += (t + te)(fh + fl)
                    const float2 pr = f2mul(t, fh);
                    const float2 pe = f2fma(t, fh, make_float2(-pr.x, -pr.y));
                    const float2 w = f2add(S, pr);
                    const float2 bq = f2sub(w, S);
                    E = f2add(E, f2add(f2add(f2sub(S, f2sub(w, bq)), f2sub(pr, bq)),
                                       f2add(pe, f2fma(t, fl, f2mul(te, fh)))));
                    S = w;
                }
            }
            // fold the two accumulators (TwoSum)
            float St, Et;
            {
                const float w = S.x + S.y;
                const float bq = w - S.x;
                Et = E.x + E.y + (S.x - (w - bq)) + (S.y - bq);
                St = w;
            }
            tc_fence_before();
            if (half == 1) s_part[eg][r] = make_float2(St, Et);
            epi_group_bar(eg);                   // TMEM and A-stage reads of this tile done, halves posted
            if (threadIdx.x == 64 + 256 * eg) {
                mbar_arrive(&sh->tmem_empty[eg]);
                mbar_arrive(&sh->empty[s]);
            }
            if (half == 0) {
                const float2 o = s_part[eg][r];
                const float w = St + o.x;
                const float bq = w - St;
                const float e = Et + o.y + (St - (w - bq)) + (o.x - bq);
                double rv = 2.0 * ((double)w + (double)e) * ldexp(1.0, 2 * ep);
                if (args.correct) {
                    // the density correction, and rho w_becke for the multipoles
                    // (the point kernel's arithmetic)
                    rv *= cf;
                    if (args.rw32) {
                        const dfl x = df_mul(df_from_bits(rv), dfl{wbh, wbl});
                        args.rw32[p] = x.h;
                        args.rw32[args.npad + p] = x.l;
                    }
                }
                rho[p] = rv;
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    const bool ok = s_fail == 0;
    if (threadIdx.x == 0) {
        for (int b = 0; b < kTcStages; ++b) {
            mbar_inval(&sh->full[b]);
            mbar_inval(&sh->empty[b]);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_inval(&sh->tmem_full[b]);
            mbar_inval(&sh->tmem_empty[b]);
        }
    }
    return ok;
}

__device__ __forceinline__ void density_tc_alloc()
{
    TcShared *sh = &tc_sh;
    if ((threadIdx.x >> 5) == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sh->tmem_base)),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
}

// after the CTA's last __syncthreads
__device__ __forceinline__ void density_tc_free(uint32_t tmem)
{
    if ((threadIdx.x >> 5) == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTcTmemCols) : "memory");
    }
}

__global__ void __launch_bounds__(kTcThreads, 1) k_density_tc(const DensTcArgs args)
{
    pdl_wait();
    density_tc_alloc();
    const uint32_t tmem = tc_sh.tmem_base;
    density_tc_cta(args, (int)blockIdx.x, (int)gridDim.x, tmem);
    density_tc_free(tmem);
    pdl_signal();
}

// the batch's grouped launch: each CTA runs items (molecule, virtual CTA) from
// the queue, TMEM allocated once for all of them
__global__ void __launch_bounds__(kTcThreads, 1) k_density_tc_group(const DensTcArgs *__restrict__ args, GroupQueue q)
{
    density_tc_alloc();
    const uint32_t tmem = tc_sh.tmem_base;
    gq_run(q, &tc_sh.item, [&](int m, int vb, int nvb) {
        const DensTcArgs a = args[m];
        return density_tc_cta(a, vb, nvb, tmem);
    });
    tc_fence_before();
    __syncthreads();
    density_tc_free(tmem);
}

// ------------------------------------------------------------------ slicing

// The slicing works on the IEEE bits with integer operations (no FP64
// arithmetic, slow on this GPU).  For x with |x| < 2^e, N = |x| 2^(30 - e)
// rounded to an integer (half away from zero), with x's sign; |N| <= 2^30.
__device__ __forceinline__ long long fixed30(unsigned long long bits, int e)
{
    const int ef = (int)((bits >> 52) & 0x7ffu);
    unsigned long long m = bits & 0xfffffffffffffull;
    int E = -1022;                               // subnormal
    if (ef != 0) {
        m |= 1ull << 52;
        E = ef - 1023;
    }
    // |x| = m 2^(E - 52), so N = m 2^-s with s = 22 + e - E >= 23 (E <= e - 1)
    const int s = 22 + e - E;
    const unsigned long long n = s > 64 ? 0ull : ((m >> (s - 1)) + 1ull) >> 1;
    return (bits >> 63) ? -(long long)n : (long long)n;
}

// exponent e with |x| < 2^e for the largest |x| given by its magnitude bits
// (frexp's exponent; 0 for zero)
__device__ __forceinline__ int exp_above(unsigned long long magbits)
{
    if (magbits == 0ull) return 0;
    const int ef = (int)(magbits >> 52);
    return ef == 0 ? -1021 : ef - 1022;
}

// N (|N| <= 2^30) -> the three FP16 slices of N 2^-22 = A_1 + A_2 + 2^-11 A_3:
// balanced digits N = d1 2^22 + d2 2^11 + d3 with |d2|, |d3| <= 2^10, so A_1 =
// d1 (|d1| <= 256), A_2 = d2 2^-11, A_3 = d3 2^-11, each exact in FP16
__device__ __forceinline__ void slice3_f16(long long N, uint16_t (&h)[kTcSlices])
{
    const long long d1 = (N + (1ll << 21)) >> 22;
    const long long r1 = N - (d1 << 22);         // [-2^21, 2^21)
    const long long d2 = (r1 + (1ll << 10)) >> 11;
    const long long d3 = r1 - (d2 << 11);        // [-2^10, 2^10)
    h[0] = __half_as_ushort(__float2half_rn((float)d1));
    h[1] = __half_as_ushort(__float2half_rn((float)d2 * 0x1p-11f));
    h[2] = __half_as_ushort(__float2half_rn((float)d3 * 0x1p-11f));
}

// Phi (FP64, [nbf][npad]) -> three FP16 slices per element in the tile layout
__global__ void k_slice_phi(int nbf, int KP, size_t npad, int ntiles, const double *__restrict__ phi,
                            __half *__restrict__ A, int *__restrict__ row_exp)
{
    const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= npad) return;
    const unsigned long long *__restrict__ pb = reinterpret_cast<const unsigned long long *>(phi);
    unsigned long long mx = 0ull;
    for (int mu = 0; mu < nbf; ++mu) mx = max(mx, pb[(size_t)mu * npad + p] & 0x7fffffffffffffffull);
    const int e = exp_above(mx);                 // every |phi| < 2^e
    row_exp[p] = e;
    const int tile = (int)(p / kTcTile), r = (int)(p % kTcTile);
    const size_t slice16 = (size_t)ntiles * kTcTile * KP / 8;     // one slice in 16-byte units
    uint4 *A16 = reinterpret_cast<uint4 *>(A);
    // eight consecutive functions (one core-matrix row) per step: one 16-byte store per slice
    for (int mu0 = 0; mu0 < KP; mu0 += 8) {
        uint32_t w[kTcSlices][4];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const int mu = mu0 + k;
            uint16_t h[kTcSlices];
            slice3_f16(mu < nbf ? fixed30(pb[(size_t)mu * npad + p], e) : 0ll, h);
#pragma unroll
            for (int i = 0; i < kTcSlices; ++i) {
                if (k & 1) w[i][k >> 1] |= (uint32_t)h[i] << 16;
                else w[i][k >> 1] = h[i];
            }
        }
        const size_t o16 = ((size_t)tile * kTcTile * KP * 2 + core_off(r, mu0, KP / 8)) / 16;
#pragma unroll
        for (int i = 0; i < kTcSlices; ++i) A16[(size_t)i * slice16 + o16] = make_uint4(w[i][0], w[i][1], w[i][2], w[i][3]);
    }
}

// P (FP64, nbf x nbf, symmetric) -> three FP16 slices per column in the B
// layout: one warp per column, lanes over the rows; with Pcopy the warp also
// copies its column of P there
// One block of the P slicing (a warp per column nu of B): the column's
// exponent and FP16 slices (and the copy of P into the context when Pcopy), and
// with S the column's share of tr(P S_grid).
__device__ __forceinline__ void slice_P_block(const SlicePArgs a, int vb)
{
    const int nbf = a.nbf, KP = a.KP, NP = a.NP;
    const double *__restrict__ P = a.P;
    uint16_t *__restrict__ B = static_cast<uint16_t *>(a.B);
    const int nu = vb * (blockDim.x >> 5) + (threadIdx.x >> 5), lane = threadIdx.x & 31;
    if (nu >= NP) return;
    const unsigned long long *__restrict__ Pb = reinterpret_cast<const unsigned long long *>(P);
    unsigned long long mx = 0ull;
    double t = 0.0;
    if (nu < nbf)
        for (int mu = lane; mu < nbf; mu += 32) {
            const unsigned long long v = Pb[(size_t)nu * nbf + mu];
            if (a.Pcopy) reinterpret_cast<unsigned long long *>(a.Pcopy)[(size_t)nu * nbf + mu] = v;
            mx = max(mx, v & 0x7fffffffffffffffull);
            if (a.S) t = fma(__longlong_as_double((long long)v), a.S[(size_t)nu * nbf + mu], t);
        }
    for (int o = 16; o > 0; o >>= 1) {
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        t += __shfl_xor_sync(0xffffffffu, t, o);
    }
    const int e = exp_above(mx);
    if (nu < nbf && lane == 0) {
        a.col_exp[nu] = e;
        if (a.S) a.tr[nu] = t;
    }
    const size_t slice = (size_t)NP * KP;
    for (int mu = lane; mu < KP; mu += 32) {
        uint16_t h[kTcSlices];
        slice3_f16((nu < nbf && mu < nbf) ? fixed30(Pb[(size_t)nu * nbf + mu], e) : 0ll, h);
        const size_t o = core_off(nu, mu, KP / 8) / 2;
        for (int i = 0; i < kTcSlices; ++i) B[(size_t)i * slice + o] = h[i];
    }
}

constexpr int kSlicePThreads = 128;

__global__ void __launch_bounds__(kSlicePThreads) k_slice_P(const SlicePArgs a)
{
    pdl_wait();
    slice_P_block(a, (int)blockIdx.x);
    pdl_signal();
}

__global__ void __launch_bounds__(kSlicePThreads) k_slice_P_group(const SlicePArgs *__restrict__ args, GroupQueue q)
{
    __shared__ int s_item;
    gq_run(q, &s_item, [&](int m, int vb, int) {
        const SlicePArgs a = args[m];
        slice_P_block(a, vb);
        return true;
    });
}

size_t density_tc_smem(int KP, int NP)
{
    return (size_t)kTcStages * kTcSlices * kTcTile * KP * 2 + (size_t)kTcSlices * NP * KP * 2 + 64;
}

bool density_tc_supported(int nbf) { return nbf <= kTcMaxK; }

// S_grid = Phi^T diag(w) Phi over the grid points, once per grid: with it
// sum_p w_p rho_p = 2 tr(P S_grid) is known from P before the density pass.
// Block b sums the pairs (mu <= nu) over points [b kSgChunk, (b + 1) kSgChunk)
// in double-float arithmetic (FP32 TwoProd / TwoSum, about 2^-44 relative; the
// FP64 pipe of this GPU is narrow) into part[b][pair] as FP64; k_sgrid_sum adds
// the blocks in order and mirrors.
constexpr int kSgThreads = 256, kSgPts = 16, kSgChunk = 1024;
constexpr int kSgTilesMax = (kTcMaxK / 2) * (kTcMaxK / 2 + 1) / 2;   // 2 x 2 tiles (I <= J)
constexpr int kSgPerThread = (kSgTilesMax + kSgThreads - 1) / kSgThreads;

// k = j (j + 1) / 2 + i, i <= j
__device__ __forceinline__ short2 tri_index(int k)
{
    int j = (int)((sqrtf(8.f * (float)k + 1.f) - 1.f) * 0.5f);
    while (j * (j + 1) / 2 > k) --j;
    while ((j + 1) * (j + 2) / 2 <= k) ++j;
    return make_short2((short)(k - j * (j + 1) / 2), (short)j);
}

// A thread takes 2 x 2 tiles (rows 2I, 2I + 1 against columns 2J, 2J + 1,
// I <= J): four loads serve four products per point.
__global__ void __launch_bounds__(kSgThreads) k_sgrid_part(int nbf, size_t npts, size_t npad,
                                                           const double *__restrict__ phi,
                                                           const double *__restrict__ w, double *__restrict__ part)
{
    __shared__ float2 sph[kTcMaxK][kSgPts + 1];     // phi as (hi, lo); rows >= nbf zero
    __shared__ float2 swph[kTcMaxK][kSgPts + 1];    // w phi as (hi, lo)
    const int npair = nbf * (nbf + 1) / 2, tid = threadIdx.x;
    const int nb2 = (nbf + 1) / 2, ntile = nb2 * (nb2 + 1) / 2;
    short2 tl[kSgPerThread];
#pragma unroll
    for (int q = 0; q < kSgPerThread; ++q) {
        const int t = tid + q * kSgThreads;
        tl[q] = t < ntile ? tri_index(t) : make_short2(0, 0);
    }
    float as[kSgPerThread][4], ae[kSgPerThread][4];
#pragma unroll
    for (int q = 0; q < kSgPerThread; ++q)
#pragma unroll
        for (int u = 0; u < 4; ++u) as[q][u] = ae[q][u] = 0.f;
    const size_t p0 = (size_t)blockIdx.x * kSgChunk, p1 = min(npts, p0 + kSgChunk);
    for (size_t s0 = p0; s0 < p1; s0 += kSgPts) {
        __syncthreads();
        for (int e = tid; e < 2 * nb2 * kSgPts; e += kSgThreads) {
            const int mu = e / kSgPts, j = e % kSgPts;
            const bool in = s0 + j < p1 && mu < nbf;
            // hi / lo split of the FP64 values with integer operations
            const dfl f = df_from_bits(in ? phi[(size_t)mu * npad + s0 + j] : 0.0);
            const dfl wf = df_mul(df_from_bits(in ? w[s0 + j] : 0.0), f);
            sph[mu][j] = make_float2(f.h, f.l);
            swph[mu][j] = make_float2(wf.h, wf.l);
        }
        __syncthreads();
#pragma unroll
        for (int q = 0; q < kSgPerThread; ++q) {
            if (tid + q * kSgThreads < ntile) {
                const int r0 = 2 * tl[q].x, c0 = 2 * tl[q].y;
#pragma unroll 4
                for (int j = 0; j < kSgPts; ++j) {
                    const float2 a0 = swph[r0][j], a1 = swph[r0 + 1][j], b0 = sph[c0][j], b1 = sph[c0 + 1][j];
                    df_mac(as[q][0], ae[q][0], a0.x, a0.y, b0.x, b0.y);
                    df_mac(as[q][1], ae[q][1], a0.x, a0.y, b1.x, b1.y);
                    df_mac(as[q][2], ae[q][2], a1.x, a1.y, b0.x, b0.y);
                    df_mac(as[q][3], ae[q][3], a1.x, a1.y, b1.x, b1.y);
                }
            }
        }
    }
#pragma unroll
    for (int q = 0; q < kSgPerThread; ++q) {
        if (tid + q * kSgThreads >= ntile) continue;
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int mu = 2 * tl[q].x + (u >> 1), nu = 2 * tl[q].y + (u & 1);
            if (mu <= nu && nu < nbf)
                part[(size_t)blockIdx.x * npair + nu * (nu + 1) / 2 + mu] = df_to(df_norm(as[q][u], ae[q][u]));
        }
    }
}

__global__ void k_sgrid_sum(int nbf, int nblk, const double *__restrict__ part, double *__restrict__ S)
{
    const int npair = nbf * (nbf + 1) / 2;
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npair) return;
    int nu = (int)((sqrtf(8.f * (float)k + 1.f) - 1.f) * 0.5f);
    while (nu * (nu + 1) / 2 > k) --nu;
    while ((nu + 1) * (nu + 2) / 2 <= k) ++nu;
    const int mu = k - nu * (nu + 1) / 2;
    double t = 0.0;
    for (int b = 0; b < nblk; ++b) t += part[(size_t)b * npair + k];
    S[(size_t)mu * nbf + nu] = t;
    S[(size_t)nu * nbf + mu] = t;
}

bool cmax_route(const dftg_ctx *c)
{
    return c->whole_build && c->d_ct_cmax && batch_group_eligible(c) && sgrid_route(c);
}

bool sgrid_route(const dftg_ctx *c)
{
    return c->d_sgrid && c->tc_ready && !c->points_only && c->cell0 == 0 && c->ncell == c->natoms &&
           (c->prec_mask & kPrecDensity) && (c->prec_mask & kPrecLda);
}

int density_tc_setup(dftg_ctx *c)
{
    if (!density_tc_supported(c->nbf)) return DFTG_OK;
    c->tc_KP = (c->nbf + 15) / 16 * 16;
    c->tc_NP = c->tc_KP;
    const int ntiles = (int)(c->npad / kTcTile);
    const size_t aslice = (size_t)ntiles * kTcTile * c->tc_KP;
    DFTG_CUDA(cudaMalloc(&c->d_tcA, sizeof(__half) * kTcSlices * aslice));
    DFTG_CUDA(cudaMalloc(&c->d_tc_rowexp, sizeof(int) * c->npad));
    DFTG_CUDA(cudaMalloc(&c->d_tcB, sizeof(__half) * kTcSlices * c->tc_NP * c->tc_KP));
    DFTG_CUDA(cudaMalloc(&c->d_tc_colexp, sizeof(int) * c->tc_NP));
    if (!c->d_flag) {
        DFTG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
    }
    k_slice_phi<<<(unsigned)((c->npad + 127) / 128), 128, 0, c->stream>>>(
        c->nbf, c->tc_KP, c->npad, ntiles, c->d_phi, reinterpret_cast<__half *>(c->d_tcA), c->d_tc_rowexp);
    DFTG_LAUNCH_CHECK();
    const size_t sm = density_tc_smem(c->tc_KP, c->tc_NP);
    (void)sm;
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density_tc), c->device));
    if (!c->points_only) {
        const int nblk = (int)((c->npts + kSgChunk - 1) / kSgChunk), npair = c->nbf * (c->nbf + 1) / 2;
        double *part = nullptr;
        DFTG_CUDA(cudaMalloc(&c->d_sgrid, sizeof(double) * (size_t)c->nbf * c->nbf));
        DFTG_CUDA(cudaMalloc(&part, sizeof(double) * (size_t)nblk * npair));
        k_sgrid_part<<<nblk, kSgThreads, 0, c->stream>>>(c->nbf, c->npts, c->npad, c->d_phi, c->d_w, part);
        cudaError_t e = cudaGetLastError();
        if (e == cudaSuccess) {
            k_sgrid_sum<<<(npair + 127) / 128, 128, 0, c->stream>>>(c->nbf, nblk, part, c->d_sgrid);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        cudaFree(part);
        if (e != cudaSuccess) return cuda_fail(e, "S_grid", __FILE__, __LINE__);
    }
    int nsm = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    c->tc_grid = nsm < ntiles ? nsm : ntiles;
    c->tc_grid_max = c->tc_grid;
    c->tc_ready = true;
    return DFTG_OK;
}

StepLaunch<SlicePArgs> step_slice_P(const dftg_ctx *c, const double *P, double *Pcopy, bool fused)
{
    StepLaunch<SlicePArgs> s;
    const bool tr = fused && sgrid_route(c);
    s.args = SlicePArgs{c->nbf, c->tc_KP, c->tc_NP, P, Pcopy, c->d_tcB, c->d_tc_colexp, tr ? c->d_sgrid : nullptr,
                        c->d_red};
    s.blocks = (c->tc_NP + kSlicePThreads / 32 - 1) / (kSlicePThreads / 32);
    s.smem = 0;
    return s;
}

StepLaunch<DensTcArgs> step_density_tc(const dftg_ctx *c, bool fused)
{
    StepLaunch<DensTcArgs> s;
    const bool correct = fused && sgrid_route(c);
    s.args = DensTcArgs{c->nbf, c->tc_KP, c->tc_NP, (int)(c->npad / kTcTile),
                        reinterpret_cast<const unsigned char *>(c->d_tcA), c->d_tc_rowexp,
                        reinterpret_cast<const unsigned char *>(c->d_tcB), c->d_tc_colexp, c->d_rho, c->d_flag,
                        correct ? 1 : 0, c->npad, c->d_scal, c->d_wsplit + 2 * c->npad,
                        correct && rw_planes(c) ? c->d_rw32 : nullptr, c->d_red, c->d_atoms, c->natoms};
    s.blocks = c->tc_grid;
    s.smem = density_tc_smem(c->tc_KP, c->tc_NP);
    return s;
}

int launch_density_tc(dftg_ctx *c, bool fused)
{
    const StepLaunch<SlicePArgs> sp = step_slice_P(c, c->d_P, nullptr, fused);
    DFTG_CUDA(launch_pdl(k_slice_P, sp.blocks, kSlicePThreads, 0, c->stream, sp.args));
    DFTG_MARK(c, "density_slices");
    const StepLaunch<DensTcArgs> dn = step_density_tc(c, fused);
    DFTG_CUDA(launch_pdl(k_density_tc, dn.blocks, kTcThreads, dn.smem, c->stream, dn.args));
    return DFTG_OK;
}

int group_slice_P(const SlicePArgs *d_args, const GroupQueue &q, int nsm, cudaStream_t st)
{
    int occ = 0;
    DFTG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_slice_P_group, kSlicePThreads, 0));
    const int grid = group_grid(q, occ, nsm);
    if (grid > 0) k_slice_P_group<<<grid, kSlicePThreads, 0, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int group_density_tc(const DensTcArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st)
{
    DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_density_tc_group), device));
    // one CTA per SM: each holds all kTcTmemCols TMEM columns for its lifetime
    const int grid = group_grid(q, 1, nsm);
    if (grid > 0) k_density_tc_group<<<grid, kTcThreads, smem, st>>>(d_args, q);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

}  // namespace dftg

// ------------------------------------------------------------------ self-test of the bounded-wait path
namespace dftg {
// one warp waits on an mbarrier that nothing arrives at; the bounded wait gives
// up after limit_ns and the kernel records code 99 in the context's flag
__global__ void k_selftest_wait(unsigned long long limit_ns, int *err)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (threadIdx.x == 0 && !mbar_wait_ns(&bar, 0u, limit_ns)) atomicExch(err, 99);
}
}  // namespace dftg

extern "C" int dftg_selftest_wait(dftg_ctx *c, double limit_ms)
{
    using namespace dftg;
    if (!c) { set_error("null context"); return DFTG_ERR_ARG; }
    if (!(limit_ms > 0.0 && limit_ms <= 2000.0)) { set_error("limit_ms %g out of (0, 2000]", limit_ms); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    if (!c->d_flag) {
        DFTG_CUDA(cudaMalloc(&c->d_flag, sizeof(int)));
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
    }
    k_selftest_wait<<<1, 32, 0, c->stream>>>((unsigned long long)(limit_ms * 1e6), c->d_flag);
    DFTG_LAUNCH_CHECK();
    return sync_scalars(c);
}
