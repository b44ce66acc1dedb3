// dftg_internal.cuh -- context layout and kernel launchers of the grid Fock build.
//
// Data layout in HBM (npad = grid size rounded up to 128; padded points carry
// zero weight and zero amplitudes so every kernel can work on whole tiles):
//   points      X, Y, Zc, W, WB, rho, V     [npad] FP64 (structure of arrays)
//   amplitudes  phi   [nbf][npad] FP64      (point-contiguous per function)
//               phi32 [nbf][npad] FP32      (mixed-precision copy)
//   point coefficients  cxc = w*v_xc, cj = w*V/2   [npad] FP64 and FP32
//   Hartree     Y [nlm][nang], rholm/U [natoms][nlm][nrad], LU factors per l,
//               spline coefficients [natoms][nlm][nrad][4] (last interval = clamp),
//               FP64 and, for the mixed path, normalised and split into FP32 hi/lo
#pragma once
#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>
#include <vector>
#include "../../include/dftg.h"

namespace dftg {

constexpr double kPi = 3.14159265358979323846;      // atomicgrid.h:50
constexpr double kPiTrunc = 3.14159265359;          // cgf.cpp:103, integrals.cpp:342
constexpr int kLmaxCap = 16;
constexpr int kMaxAtoms = 256;
constexpr int kPtsAlign = 128;
constexpr int kMaxRedCtas = 1024;    // CTAs of a persistent kernel that writes per-CTA reduction partials

void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define DFTG_CUDA(call)                                                        \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return ::dftg::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define DFTG_LAUNCH_CHECK() DFTG_CUDA(cudaGetLastError())
#define DFTG_TRY_L(x) do { int rc_l_ = (x); if (rc_l_ != DFTG_OK) return rc_l_; } while (0)

// Programmatic dependent launch between the kernels of one build: each kernel
// waits for its predecessors' completion and memory first (griddepcontrol.wait,
// a no-op for a launch without a programmatic dependency) and signals at its end,
// so the successor's launch overlaps the tail of the predecessor.
#if defined(__CUDACC__)
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_signal() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
#endif
template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*k)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t st,
                              const Args &...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, k, args...);
}

// compensated FP32 accumulation (Knuth's TwoSum): s + e is the running sum
__device__ __forceinline__ void two_sum_acc(float &s, float &e, float x)
{
    const float t = s + x;
    const float bp = t - s;
    e += (s - (t - bp)) + (x - bp);
    s = t;
}

// Fold the maximum of non-negative v over the lanes of a warp that share a
// chunk into cmax[chunk], one atomicMax per (warp, chunk): the IEEE bits of
// non-negative floats order like their values, and a maximum is exact and
// independent of order.  Every lane of the warp calls it; chunk < 0 for a lane
// without a value.
__device__ __forceinline__ void warp_chunk_max(unsigned *cmax, int chunk, float v)
{
    const unsigned grp = __match_any_sync(0xffffffffu, chunk);
    const unsigned m = __reduce_max_sync(grp, __float_as_uint(v));
    if (chunk >= 0 && (int)(threadIdx.x & 31) == __ffs(grp) - 1) atomicMax(cmax + chunk, m);
}

// Packed FP32 pairs: one instruction for two independent lanes, each rounded to
// nearest exactly as the scalar operation (and, being explicit roundings, never
// contracted into an FMA, so error-free transformations keep their meaning).
__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b)
{
    unsigned long long d;
    asm("sub.rn.f32x2 %0, %1, %2;"
        : "=l"(d)
        : "l"(*reinterpret_cast<const unsigned long long *>(&a)), "l"(*reinterpret_cast<const unsigned long long *>(&b)));
    return *reinterpret_cast<const float2 *>(&d);
}

// Double-float arithmetic (value = h + l, |l| <= ulp(h) / 2): about 48-bit
// precision from FP32 operations, for per-build loops that would otherwise run
// in FP64 (slow on this GPU).  TwoSum / TwoProd with fmaf (Dekker, Knuth).
struct dfl {
    float h, l;
};
__device__ __forceinline__ dfl df_norm(float s, float e)
{
    const float h = s + e;
    return {h, e - (h - s)};
}
__device__ __forceinline__ dfl df_add(dfl a, dfl b)
{
    const float s = a.h + b.h;
    const float bp = s - a.h;
    const float e = (a.h - (s - bp)) + (b.h - bp) + a.l + b.l;
    return df_norm(s, e);
}
__device__ __forceinline__ dfl df_neg(dfl a) { return {-a.h, -a.l}; }
__device__ __forceinline__ dfl df_sub(dfl a, dfl b) { return df_add(a, df_neg(b)); }
__device__ __forceinline__ dfl df_mul(dfl a, dfl b)
{
    const float p = a.h * b.h;
    const float e = fmaf(a.h, b.h, -p) + (a.h * b.l + a.l * b.h);
    return df_norm(p, e);
}
__device__ __forceinline__ dfl df_fma(dfl acc, dfl a, dfl b) { return df_add(acc, df_mul(a, b)); }
// s + e += (ah + al)(bh + bl): the leading product exact (TwoProd), the sum
// compensated (TwoSum), the cross terms and roundings gathered in e
__device__ __forceinline__ void df_mac(float &s, float &e, float ah, float al, float bh, float bl)
{
    const float p = ah * bh;
    const float pe = fmaf(ah, bh, -p);
    const float t = s + p;
    const float bp = t - s;
    e += ((s - (t - bp)) + (p - bp)) + fmaf(ah, bl, fmaf(al, bh, pe));
    s = t;
}

__host__ __device__ __forceinline__ dfl df_from(double x)
{
    const float h = (float)x;
    return {h, (float)(x - (double)h)};
}
__device__ __forceinline__ double df_to(dfl a) { return (double)a.h + (double)a.l; }

// x as a double-float from its IEEE bits with integer operations (no FP64
// arithmetic): h = x rounded to 24 bits (half away from zero), l = the
// remainder rounded to FP32.  |x| < 2^-100 gives 0; |x| < 2^127.
__device__ __forceinline__ dfl df_from_bits(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ef = (int)((b >> 52) & 0x7ffu);
    if (ef < 1023 - 100) return {0.f, 0.f};
    const unsigned sgn = (unsigned)(b >> 32) & 0x80000000u;
    const long long m = (long long)((b & 0xfffffffffffffull) | (1ull << 52));   // x = m 2^(E - 52)
    const long long mh = (m + (1ll << 28)) >> 29;                               // [2^23, 2^24]
    const int rem = (int)(m - (mh << 29));                                      // [-2^28, 2^28]
    const int E = ef - 1023;
    // h = mh 2^(E - 23); mh = 2^24 is 2^(E + 1)
    const float h = __uint_as_float(sgn | ((unsigned)(E + 127 + (int)(mh >> 24)) << 23) | ((unsigned)mh & 0x7fffffu));
    const float l = (float)rem * 0x1p-52f * __int_as_float((127 + E) << 23);
    return {h, sgn ? -l : l};
}

// Deterministic sum of v over the block (blockDim.x a multiple of 32, at most
// 1024): butterfly shuffles inside each warp, then warp totals in warp order.
// The result is valid in thread 0.  sh: 32 doubles of shared memory.
__device__ __forceinline__ double block_sum(double v, double *sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    __syncthreads();
    return s;
}

// True in exactly one of nblocks blocks: the last to get here.  Every block's
// global writes made before the call are visible to that block (read them with
// __ldcg).  The counter is reset for the next launch.
__device__ __forceinline__ bool last_block_of(int *counter, int nblocks, int *s_flag)
{
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        const int t = atomicAdd(counter, 1);
        *s_flag = (t == nblocks - 1) ? 1 : 0;
        if (*s_flag) *counter = 0;
    }
    __syncthreads();
    if (*s_flag) __threadfence();
    return *s_flag != 0;
}

// ---------------------------------------------------------------- grouped launches
// A batch of molecules runs each step of the build as one persistent launch.
// The launch's work items 0 .. nitems - 1 are the blocks of the molecules' own
// launches, molecule-major: item i belongs to molecule m with prefix[m] <= i <
// prefix[m + 1] and is its block vb = i - prefix[m] of nvb = prefix[m + 1] -
// prefix[m].  Every CTA takes `take` consecutive items at a time from a device
// counter (zero at the start of the launch) until none are left, and runs each
// item as that block of the molecule's own launch, so each molecule's
// arithmetic and reduction order are those of its single build.
struct GroupQueue {
    const int *prefix;    // [nmol + 1], non-decreasing, prefix[0] = 0, prefix[nmol] = nitems
    int nmol, nitems, take;
    int *head;            // items handed out so far
};

// molecule of item i: the largest m < nmol with prefix[m] <= i (its range holds i)
__device__ __forceinline__ int gq_molecule(const GroupQueue &q, int i)
{
    int lo = 0, hi = q.nmol - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(q.prefix + mid) <= i) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// The CTA's item loop: f(m, vb, nvb) runs one item with every thread of the
// CTA and returns false to stop the CTA (a bounded wait that gave up).  s_item:
// one int of shared memory.
template <typename F>
__device__ __forceinline__ void gq_run(const GroupQueue &q, int *s_item, F &&f)
{
    for (;;) {
        __syncthreads();                        // the previous item is done with shared memory and s_item
        if (threadIdx.x == 0) *s_item = atomicAdd(q.head, q.take);
        __syncthreads();
        const int i0 = *s_item;
        if (i0 >= q.nitems) return;
        const int i1 = min(q.nitems, i0 + q.take);
        for (int i = i0; i < i1; ++i) {
            const int m = gq_molecule(q, i);
            const int b0 = __ldg(q.prefix + m);
            if (i > i0) __syncthreads();
            if (!f(m, i - b0, __ldg(q.prefix + m + 1) - b0)) return;
        }
    }
}

__device__ __forceinline__ unsigned long long globaltimer_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}

// *flag = v with release semantics at GPU scope (after the caller's writes)
__device__ __forceinline__ void flag_release(int *flag, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(flag), "r"(v) : "memory");
}

// Bounded wait of the CTA until *flag >= v: thread 0 polls with acquire loads,
// gives up after limit_ns of wall-clock time (or 2^26 polls whatever the
// timer).  Block-uniform result; s_ok: one int of shared memory.
__device__ __forceinline__ bool wait_flag_ge(const int *flag, int v, unsigned long long limit_ns, int *s_ok)
{
    if (threadIdx.x == 0) {
        int ok = 0;
        const unsigned long long t0 = globaltimer_ns();
        for (unsigned it = 0; it < (1u << 26); ++it) {
            int cur;
            asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(cur) : "l"(flag) : "memory");
            if (cur >= v) { ok = 1; break; }
            if ((it & 15u) == 0u && globaltimer_ns() - t0 > limit_ns) break;
            __nanosleep(128);
        }
        *s_ok = ok;
    }
    __syncthreads();
    return *s_ok != 0;
}

// True in exactly one block: the last to get here.  Every block's global writes
// made before the call are visible to that block (read them with __ldcg).  The
// counter is reset for the next launch.
__device__ __forceinline__ bool last_block(int *counter, int *s_flag)
{
    return last_block_of(counter, (int)gridDim.x, s_flag);
}

// counters of the last-block reductions
enum { kCntAtoms = 0, kCntLda = 1, kCntEJ = 2, kNumCounters = 4 };

}  // namespace dftg

struct dftg_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int precision = DFTG_PREC_FP64;
    unsigned prec_mask = 0;       // kPrec* bits: steps run in reduced precision

    // molecule and basis (host copies)
    int natoms = 0, nbf = 0, nprim = 0;
    std::vector<int> Z;
    std::vector<double> xyz;
    std::vector<int> bf_atom, bf_lmn, bf_off;
    std::vector<double> alpha, coef, norm;

    // grid: the fuzzy cells of atoms cell0 .. cell0 + ncell - 1 (every atom's
    // cell unless the context is one shard of an atom-cell partition)
    int cell0 = 0, ncell = 0;
    int nrad = 0, leb = 0, nang = 0, lmax = 0, nlm = 0;
    size_t npts = 0, npad = 0;
    std::vector<double> r_n, w_rad;

    // device: geometry and basis
    double *d_atoms = nullptr;    // [natoms][4] x y z Z
    double *d_rab = nullptr;      // [natoms][natoms] inter-atomic distances
    double *d_rn = nullptr;       // [nrad]
    double *d_wrad = nullptr;     // [nrad]
    double *d_leb = nullptr;      // [nang][4]
    int *d_bf_lmn = nullptr;      // [nbf][3]
    int *d_bf_off = nullptr;      // [nbf+1]
    int *d_bf_atom = nullptr;     // [nbf]
    double *d_pa = nullptr;       // [nprim] exponents
    double *d_pcn = nullptr;      // [nprim] coefficient * normalisation

    // device: per point
    double *d_x = nullptr, *d_y = nullptr, *d_z = nullptr;
    double *d_w = nullptr, *d_wb = nullptr;
    double *d_rho = nullptr, *d_V = nullptr, *d_Vown = nullptr;
    double *d_invr = nullptr;     // [npts] 1 / distance to the owning atom
    double *d_cxc = nullptr, *d_cj = nullptr;
    float *d_cxc32 = nullptr, *d_cj32 = nullptr;
    double *d_phi = nullptr;
    float *d_phi32 = nullptr;

    // device: matrices
    double *d_P = nullptr;
    float *d_P32 = nullptr;       // [2][nbf][ldp] FP32 hi and lo of P, ldp = nbf rounded up to 4 (mixed CUDA-core density)
    double *d_J = nullptr, *d_XC = nullptr;
    double *d_part = nullptr;     // contraction partials [nchunk][2][nbf][nbf]
    size_t part_elems = 0;
    int nchunk = 0;               // point chunks of the contraction
    int ntiles = 0;               // output blocks on or above the diagonal
    void *d_tiles = nullptr;      // [ntiles] int2 block coordinates
    double *d_sgrid = nullptr;    // [nbf][nbf] S_grid = Phi^T diag(w) Phi (FP64), for the correction factor
    double *d_red = nullptr;      // reduction partials
    size_t red_elems = 0;
    size_t red_lda_off = 0;       // the LDA point kernel's partials start here (it may run beside the Hartree steps)
    cudaStream_t aux_stream = nullptr;          // the second branch of the whole build
    bool whole_build = false;     // set while the whole build's launches (or a batch's records) are made
    unsigned *d_ct_cmax = nullptr;   // [2][nchunk] max |c / w| bits per contraction chunk (XC, J), zero between builds
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    double *d_scal = nullptr;     // scalars, see kScal* below
    int *d_counters = nullptr;    // [kNumCounters] last-block counters (zero between launches)
    float *d_wsplit = nullptr;    // [4][npad] w and w_becke as FP32 hi / lo planes (mixed point kernel)
    int2 *d_lebpair = nullptr;    // [nang / 2] Lebedev directions paired with their antipodes
    int nlebpair = 0;
    double *h_scal = nullptr;     // pinned host mirror of d_scal

    // device: Hartree
    double *d_Y = nullptr;        // [nlm][nang] Y_lm of the Lebedev directions
    double *d_Yw = nullptr;       // [nlm][nang] w_leb * Y_lm
    double *d_pre = nullptr;      // [nlm] spherical-harmonic prefactors
    float *d_pre32 = nullptr;
    double *d_rec = nullptr;      // [nlm][2] associated-Legendre recursion coefficients
    float *d_rec32 = nullptr;
    double *d_rholm = nullptr;    // [natoms][nlm][nrad] (FP64 path)
    double *d_U = nullptr;        // [natoms][nlm][nrad]
    float *d_U32 = nullptr;       // [2][natoms][nlm][nrad] U split into FP32 hi, lo
    float *d_U32T = nullptr;      // [2][natoms][nrad][nlm] the same, transposed
    float *d_Y32 = nullptr;       // [2][nlm][nang] Y_lm split into FP32 hi, lo
    float *d_Ywt32 = nullptr;     // [2][nang][nlm] w_leb Y_lm split, transposed
    double *d_fold = nullptr;     // [nlm] Y_lm normalisation of the integer recursion
    double *d_Gt = nullptr;       // [lmax+1][nrad (k)][nrad (i)] radial Poisson solution map
    double *d_Gb = nullptr;       // [nrad] boundary column of the l = 0 map (times q_a)
    double *d_Kt = nullptr;       // [nrad (j)][nrad (i)] spline derivative map
    float *d_maps32 = nullptr;    // double-float (hi block, lo block) copies of Gt, Gb, Kt, 1/h, fold
    size_t npairs = 0;            // (point, other atom) pairs of the cross-atom potential
    void *d_pairs = nullptr;      // [npairs] float4 (unit vector, 1/r) then [npairs] float2 (t, k << 16 | interval),
                                  // ordered by (atom, spline interval)
    void *d_cross_tasks = nullptr; // [ncross_tasks] int4 (first pair, pairs, atom, interval)
    int ncross_tasks = 0;
    int *d_pairpos = nullptr;     // [npts][natoms] place of pair (p, k) in d_pairs
    void *d_pairv = nullptr;      // [npairs] float2 contributions
    double *d_sx = nullptr;       // [nrad] increasing spline abscissae
    double *d_splf = nullptr;     // spline factorisation (x only)
    double *d_spl = nullptr;      // [natoms][nlm][nrad][4] FP64 spline coefficients
    float *d_splm = nullptr;      // [natoms][nlm][nrad][8] normalised coefficients, FP32 hi + lo

    // device: tensor-core density (integer-slice split of phi and P)
    bool tc_ready = false;
    int tc_KP = 0, tc_NP = 0, tc_grid = 0;
    void *d_tcA = nullptr;        // [3][tiles][128 x KP] FP16 slices of phi
    void *d_tcB = nullptr;        // [3][NP x KP] FP16 slices of P
    int *d_tc_rowexp = nullptr;   // [npad] per-point scale exponents
    int *d_tc_colexp = nullptr;   // [NP] per-column scale exponents of P
    float *d_rw32 = nullptr;      // [2][npad] rho w_becke split into FP32 hi, lo (mixed multipole input)
    bool rw_ready = false;        // d_rw32 holds the current corrected rho (written by the point kernel)
    int *d_flag = nullptr;        // device error flag (bounded waits that expired)

    // device: tensor-core density for 81 <= nbf <= 1024 (128-point tiles x 128-column blocks)
    bool dt_ready = false;
    int dt_nks = 0, dt_nnb = 0, dt_grid = 0;
    void *d_dt_A = nullptr;       // [tiles][K stages][4][128 x 32] BF16 slices of phi (set-up)
    void *d_dt_B = nullptr;       // [column blocks][K stages][4][128 x 32] BF16 slices of P (every build)
    int *d_dt_exp = nullptr;      // [npad] point exponents, then [blocks x 128] column exponents

    // device: tensor-core XC / J contraction (split-K over point chunks)
    bool ct_ready = false;
    int ct_NP = 0, ct_AR = 0, ct_nst = 0, ct_spart = 0, ct_nkb = 0, ct_kbpc = 0, ct_nchunk = 0, ct_grid = 0;
    int *d_ct_rowexp = nullptr;   // [2][nchunk][nbf] exponent bounds of |phi| and |w phi| per point
                                  // chunk, then [nchunk] int2 bounds of |c_xc / w|, |c_j / w| (per build)
    float *d_ct_winv = nullptr;   // [npad] 1 / w (0 where w vanishes)
    void *d_ct_A = nullptr;       // [nkb][3][AR x 32] BF16 slices of phi, shared-memory operand layout

    // device: tiled tensor-core contraction for 128 < nbf <= 1024 (128 x 128 tiles of
    // the upper block triangle, split-K over point chunks, one pass per matrix)
    bool tt_ready = false;
    int tt_AR = 0, tt_nkb = 0, tt_kbpc = 0, tt_nchunk = 0, tt_ntiles = 0, tt_ksplit = 0, tt_grid = 0;
    int *d_tt_exp = nullptr;      // [2][nchunk][nbf] exponent bounds of |phi|, |w phi|, then [nchunk] int2 of |c / w|
    float *d_tt_winv = nullptr;   // [npad] 1 / w (0 where w vanishes)
    void *d_tt_A = nullptr;       // [nkb][3][AR x 32] BF16 slices of phi (set-up)
    void *d_tt_B = nullptr;       // [nkb][3][AR x 32] BF16 slices of c phi (every pass)
    void *d_tt_part = nullptr;    // [grid][128 x 128] double-float CTA partials

    // device: one-electron integrals output (allocated on first use)
    double *d_ints_work = nullptr;

    // backward pass (allocated on first use)
    bool bw_ready = false;
    int bw_nb_phi = 0, bw_nb_becke = 0, bw_nb_cross = 0, bw_nb_cross32 = 0;   // partial rows of the force kernels
    float *d_bw_geo = nullptr;    // FP32 1 / R_Bk [natoms^2] (padded to 4), then [natoms^2][4] (R_B - R_k) / R_Bk
    double *d_bw_geo64 = nullptr; // the same in FP64
    int bw_geo_off = 0;           // element offset of the unit-vector table
    double *d_bw_pt = nullptr;    // [7][npad] u, mbar, g, e, h, 2h, dE/dwb
    double *d_bw_lm = nullptr;    // Ubar, rbar [natoms][nlm][nrad], qbar [natoms], scalars [8], block sums
    double *d_bw_fpart = nullptr; // [rows][natoms][3] per-block force partials
    double *d_bw_out = nullptr;   // dE/dP [nbf][nbf], dE/dR [natoms][3]
    int *d_bw_counter = nullptr;  // last-block counter of the gamma reduction
    int *d_bw_pairp = nullptr;    // [npairs] grid point of each sorted pair
    int *d_bw_binfirst = nullptr; // [natoms * nrad + 1] first task of each (atom, interval) bin
    double *d_bw_cpart = nullptr; // [ncross_tasks][nlm][4] transposed cross-atom partials
    float *d_bw_prim32 = nullptr; // FP32 primitive exponents [nprim] then coefficients [nprim]
    bool have_build = false;      // a complete build left rho, V and the scalars on the device
    unsigned fwd_mask = 0;        // precision mask of that build (the backward follows it)

    bool points_only = false;     // built from explicit points and function centres: no cells, no Hartree
    int shard_phase = 0;          // atom-cell shard build: 1 after the density, 2 after the multipoles

    // call-order state
    bool have_density = false;
    bool have_hartree = false;
    bool rho_scaled = false;      // rho on the device carries the correction factor

    // launch shapes of the tensor-core kernels (CTAs, contraction stages): set
    // up at the largest that fits, lowered by the autotuner
    int tc_grid_max = 0, ct_grid_max = 0, ct_nst_max = 0, ct_nst_min = 0;

    // CUDA graph of the per-build kernel sequence (keyed by precision mask, stream and launch shapes)
    cudaGraphExec_t pipe_exec = nullptr;
    int pipe_shape[3] = {0, 0, 0};
    unsigned pipe_mask = 0;
    cudaStream_t pipe_stream = nullptr;
    bool pipe_warm = false;

    // device SCF driver (k_scf.cu), created by dftg_scf_init
    struct dftg_scf_state *scf = nullptr;

    // per-phase CUDA-event timing (dftg_fock_build_profile)
    static constexpr int kMaxMarks = 24;
    cudaEvent_t prof_ev[kMaxMarks] = {};
    const char *prof_name[kMaxMarks] = {};
    int prof_n = 0;
    bool prof_on = false;
};

namespace dftg {

// steps of the build that the mixed path runs in split / single precision
enum {
    kPrecDensity = 1,     // rho = 2 phi^T P phi
    kPrecLda = 2,         // point kernel
    kPrecMultipole = 4,   // rho_lm projection and own-cell potential
    kPrecCross = 8,       // cross-atom potential
    kPrecContract = 16,   // XC and J contractions
    kPrecAll = 31,
};

// scalar slots in d_scal
enum {
    kScalSum = 0,      // sum_p w rho (before correction)
    kScalScale = 1,    // correction factor
    kScalExc = 2,      // E_xc
    kScalNelec = 3,    // integral of corrected rho
    kScalEJ = 4,       // E_J = 2 tr(P J) = sum_p (w V / 2) rho_raw, FP64 on the grid
    kScalAtomQ = 8,    // [natoms] per-atom integral of rho (after correction)
};
inline size_t scal_elems(int natoms) { return 8 + (size_t)natoms; }

// CTAs of a grouped launch: every CTA resident (occ per SM on nsm SMs), and no
// more than the queue has runs of items
inline int group_grid(const GroupQueue &q, int occ, int nsm)
{
    const int runs = (q.nitems + q.take - 1) / q.take;
    const int resident = (occ > 0 ? occ : 1) * nsm;
    return runs < resident ? runs : resident;
}

// ---------------------------------------------------------------- steps of the mixed build
// The arguments of one molecule's launch of each step, as one record: the
// single build passes it by value, a batch's grouped launch reads molecule m's
// record from a device array (one per molecule).
struct SlicePArgs {            // P -> FP16 slices (density operand)
    int nbf, KP, NP;
    const double *P;
    double *Pcopy;             // also copies P here when not null (the context's own P)
    void *B;
    int *col_exp;
    const double *S;           // when not null: tr[nu] = sum_mu P[nu][mu] S_grid[nu][mu]
    double *tr;
};
struct DensTcArgs {            // rho on the tensor cores
    int nbf, KP, NP, ntiles;
    const unsigned char *A;
    const int *row_exp;
    const unsigned char *B;
    const int *col_exp;
    double *rho;
    int *err;
    // correct: rho times the correction factor sum Z / (2 tr(P S_grid)), formed by
    // the epilogue warps of every CTA before their first tile from the P-slicing
    // step's column partials (block 0 writes it and the total to scal), and the
    // rho w_becke hi / lo planes into rw32 when not null
    int correct;
    size_t npad;
    double *scal;
    const float *wb2;          // [2][npad] FP32 hi / lo planes of w_becke
    float *rw32;
    const double *tr;          // [nbf] column partials of tr(P S_grid) (the P-slicing step)
    const double *atoms;       // [natoms][4]: x, y, z, Z
    int natoms;
};
struct SumsArgs {              // per-atom sums of w rho, correction factor
    size_t per_atom;
    int cpa, natoms, mode;
    const double *w, *rho;
    double *part;
    const double *atoms;
    double *scal;
    int *counter;
    int *done;                 // set to 1 by the last block once scal is written (grouped launch), or null
};
struct LdaArgs {               // LDA point kernel
    size_t npad;
    double *rho;
    const double *w;
    double *scal;
    int apply_scale, want64, want_n;
    double *cxc;
    float *cxc32;
    double *part;
    int *counter;
    const double *wb;
    float *rw32;
    const float *w2, *wb2;     // w and w_becke as FP32 hi / lo planes [2][npad] (mixed kernel)
    // when cmax is not null: max |cxc32 / w| per contraction chunk of chunk_pts
    // points into cmax (the contraction's coefficient bounds, no separate pass)
    unsigned *cmax;
    const float *winv;
    int chunk_pts;
};
struct MpArgs {                // multipole chain of one atom cell per (cell, l group)
    int natoms, cell0, N, nang, lmax, ngroup, want64;
    const float *rw32;
    size_t npad;
    const double *rho, *wb, *w;
    const float *Ywt32, *maps;
    double *scal, *U;
    float *U32, *U32T;
    double *spl;
    float *splm;
    const int2 *pairs;         // [npair] Lebedev directions (j, antipode of j), j < antipode
    int npair;
};
struct VcbArgs {               // cross-atom pair contributions, one block per bin task
    int nrad, lmax;
    const int4 *tasks;
    const float4 *pgeo;
    const float2 *ptk;
    const float *splm;
    float2 *out;
};
struct GoArgs {                // own-cell potential + pair sums per point, cj, E_J
    size_t npts, npad, uhalf;
    int natoms, cell0, nrad, nang, nlm, nslab, nsplit, scaled;
    const int *pos;
    const float2 *pairv;
    const float *U32T, *Y32;
    const double *invr, *W, *rho;
    double *V, *cj;
    float *cj32;
    double *part, *scal;
    int *counter;
    const int2 *pairs;         // [npair] Lebedev directions (j, antipode of j)
    int npair;
    unsigned *cmax;            // max |cj32 / w| per contraction chunk, or null
    const float *winv;
    int chunk_pts;
};
struct CexpArgs {              // per-chunk exponent bounds of the point coefficients
    int nkb, kbpc;
    const float *cxc, *cj, *winv;
    int2 *cexp;
};
struct CtArgs {                // XC and J contraction on the tensor cores
    int nbf, AR, NP, nst, spart, nkb, kbpc, nchunk;
    const unsigned char *aslices;
    const int *rowexp, *swexp;
    const int2 *cexp;
    const float *cxc, *cj;
    float2 *part;
    int *err;
    const unsigned *cmax;      // when not null: [2][nchunk] max |c / w| bits (the bounds' source instead of cexp)
};
struct SumsLdaCtl {            // the batch's fused atom-sum + point-kernel launch
    int *head;                 // one queue over both item ranges
    int *done;                 // [nmol] set by each molecule's last atom-sum block
    int *err;                  // code 21 when a wait gave up
    unsigned long long limit_ns;
    int stall_mol;             // -1, or the molecule whose waits cannot end (self-test)
};
// one molecule's launch of a step: its arguments, blocks and dynamic shared memory
template <typename A>
struct StepLaunch {
    A args;
    int blocks = 0;
    size_t smem = 0;
};
struct RedArgs {               // sum of the contraction partials, symmetric XC and J
    int nbf, nparts, want_xc, want_j;
    const float2 *part;
    double *XC, *J;
    double *XC2, *J2;          // second copies (a batch's output buffers), or null
    const double *scal;        // with sc: copy E_xc, N, E_J to sc[0..2] (block 0)
    double *sc;
    unsigned *cmax;            // when not null: block 0 clears [ncmax] for the next build
    int ncmax;
};

// Raise a kernel's dynamic shared-memory limit to the device maximum (minus
// its static shared memory), once per kernel and device.  The limit is a
// property of the function, shared by every context, so it is never lowered.
int allow_max_dyn_smem(const void *func, int device);

// records a named event after the preceding launch when profiling is on
int mark(dftg_ctx *c, const char *name);
#define DFTG_MARK(c, name) do { if ((c)->prof_on) { int rc_m_ = ::dftg::mark((c), (name)); if (rc_m_) return rc_m_; } } while (0)

// k_grid.cu
int launch_grid(dftg_ctx *c);
int launch_amplitudes(dftg_ctx *c);
// k_density.cu
// fused: the whole build's form on the S_grid route (the density epilogue forms
// the correction factor from 2 tr(P S_grid), applies it and writes the rho
// w_becke planes; no atom-sum pass)
int launch_density(dftg_ctx *c, bool fused = false);
enum { kSumsOnly = 0, kSumsCorrect = 1, kSumsFactor = 2 };
// k_density_tc.cu
int density_tc_setup(dftg_ctx *c);
// the mixed build takes the density correction's total from 2 tr(P S_grid)
// in the density pass (no atom-sum pass)
bool sgrid_route(const dftg_ctx *c);
// the whole mixed build takes the contraction's coefficient bounds from the
// point kernel and the potential gather (atomic chunk maxima), no bounds pass
bool cmax_route(const dftg_ctx *c);
int launch_density_tc(dftg_ctx *c, bool fused);
// k_density_tt.cu
int density_tt_setup(dftg_ctx *c);
int launch_density_tt(dftg_ctx *c);
int launch_atom_sums(dftg_ctx *c, int mode);
// write_rw: the point kernel also writes the rho w_becke planes (when the
// multipoles take them)
int launch_xc_points(dftg_ctx *c, bool apply_scale, bool with_n = false, bool write_rw = true);
// the rho w_becke planes exist and the multipole step takes them
bool rw_planes(const dftg_ctx *c);
int launch_weight_planes(dftg_ctx *c);
// k_hartree.cu
int hartree_setup(dftg_ctx *c);
int cross_pairs_setup(dftg_ctx *c);
size_t hartree_splf_elems(int nrad);
int launch_hartree(dftg_ctx *c);
int launch_hartree_multipoles(dftg_ctx *c);
int launch_hartree_cross(dftg_ctx *c);
// k_adjoint.cu
int launch_backward(dftg_ctx *c, double sxc, double sj, double *dEdP_dev, double *dEdR_dev);
// k_integrals.cu
int launch_one_electron(dftg_ctx *c, double *dS, double *dT, double *dV);
// dftg_capi.cu: one build on d_P (raw launches, capturable), the same through the
// context's cached graph, and the host read of the scalars + bounded-wait flag
int fock_pipeline(dftg_ctx *c);
int fock_pipeline_graph(dftg_ctx *c);
int sync_scalars(dftg_ctx *c);
// k_scf.cu
void scf_free(dftg_ctx *c);
// k_contract.cu
int contract_setup(dftg_ctx *c);
size_t contract_part_elems(int nbf, size_t npad);
size_t reduction_elems(size_t npad, int natoms, int nrad, int nang);
size_t lda_blocks(size_t npad);   // blocks of the LDA point kernel
int launch_contract(dftg_ctx *c, bool want_xc, bool want_j);
int launch_contract_coef(dftg_ctx *c, const double *coef, double *out);
int launch_contract_coef32(dftg_ctx *c, const float *coef, double *out);
// k_contract_tc.cu
size_t contract_tc_part_elems(int nbf, size_t npad, int nsm);
int contract_tc_setup(dftg_ctx *c);
int launch_contract_tc(dftg_ctx *c);
int launch_contract_tc_reduce(dftg_ctx *c, bool want_xc, bool want_j);
int launch_contract_tc_on(dftg_ctx *c, const float *cxc32, const float *cj32);
int launch_contract_tc_reduce_to(dftg_ctx *c, bool want_xc, bool want_j, double *XC, double *J);
int ct_setup_tables(dftg_ctx *c, int AR, int nkb, int kbpc, int nchunk, int *rowexp, int *swexp, float *winv,
                    void *A);
int ct_launch_cexp(dftg_ctx *c, int nkb, int kbpc, int nchunk, const float *cx, const float *cy, const float *winv,
                   int2 *cexp);
// One molecule's launch of each step of the mixed build (its arguments, blocks
// and shared memory; the single build launches exactly these), and the batch's
// grouped launch of each step over all molecules (device argument arrays, one
// queue per launch).
StepLaunch<SlicePArgs> step_slice_P(const dftg_ctx *c, const double *P, double *Pcopy, bool fused);
StepLaunch<DensTcArgs> step_density_tc(const dftg_ctx *c, bool fused);
StepLaunch<SumsArgs> step_atom_sums(const dftg_ctx *c, int mode);
StepLaunch<LdaArgs> step_lda(const dftg_ctx *c, bool apply_scale, bool with_n, bool write_rw);
StepLaunch<MpArgs> step_multipole(const dftg_ctx *c, bool rw_ready);
StepLaunch<VcbArgs> step_vcross_bins(const dftg_ctx *c);
StepLaunch<GoArgs> step_gather_own(const dftg_ctx *c, bool rho_scaled);
StepLaunch<CexpArgs> step_cexp(const dftg_ctx *c, const float *cx, const float *cy);
StepLaunch<CtArgs> step_contract_tc(const dftg_ctx *c, const float *cx, const float *cy);
StepLaunch<RedArgs> step_contract_reduce(const dftg_ctx *c, bool want_xc, bool want_j, double *XC, double *J);
int group_slice_P(const SlicePArgs *d_args, const GroupQueue &q, int nsm, cudaStream_t st);
int group_density_tc(const DensTcArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st);
int group_sums_lda(const SumsArgs *d_sums, const GroupQueue &qs, const LdaArgs *d_lda, const GroupQueue &ql,
                   const SumsLdaCtl &ctl, int nsm, cudaStream_t st);
int group_multipole(const MpArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st);
int group_vcross_bins(const VcbArgs *d_args, const GroupQueue &q, int lmax, size_t smem, int nsm, cudaStream_t st);
int group_gather_own(const GoArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st);
int group_cexp(const CexpArgs *d_args, const GroupQueue &q, int nsm, cudaStream_t st);
int group_contract_tc(const CtArgs *d_args, const GroupQueue &q, size_t smem, int device, int nsm, cudaStream_t st);
int group_contract_reduce(const RedArgs *d_args, const GroupQueue &q, int nsm, cudaStream_t st);
// k_batch.cu: the persistent launches of a batch of mixed builds
struct BatchPlan;
bool batch_group_eligible(const dftg_ctx *c);
int batch_plan_create(dftg_ctx *const *ctx, int n, const double *const *P, double *const *J, double *const *XC,
                      double *const *sc, BatchPlan **out);
void batch_plan_free(BatchPlan *bp);
int batch_plan_enqueue(const BatchPlan *bp, cudaStream_t st, int stall_mol, unsigned long long limit_ns,
                       bool sums_lda_only);
int batch_plan_take_error(const BatchPlan *bp, cudaStream_t st, int *code);
// k_contract_tt.cu
int contract_tt_setup(dftg_ctx *c);
int launch_contract_tt_bounds(dftg_ctx *c, const float *cx, const float *cy);
int launch_contract_tt(dftg_ctx *c, const float *coef, int which, double *out);

}  // namespace dftg
