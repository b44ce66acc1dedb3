// k_contract.cu -- K4: XC = phi^T diag(w v_xc) phi and J = phi^T diag(w V / 2) phi
// in one pass over the amplitudes (dft.cpp:424-432, atomicgrid.cpp:471-488).
//
// CUDA-core form.  The nbf x nbf output is cut into TILE x TILE blocks
// (TILE = 16 R); only blocks on or above the diagonal are computed, the rest is
// mirrored.  The point dimension is split into nchunk contiguous chunks (split-K):
// CTA (tile, chunk) accumulates its chunk in registers (R x R outputs of each
// matrix per thread) and stores an FP64 partial; a second kernel sums the
// partials of each element in chunk order (deterministic FP64 reduction).
// T = double for the FP64 path, float for the mixed path (FP32 products, FP32
// sums per 32-point stage carried across stages as TwoSum pairs, FP64 across
// chunks).
#include <vector>
#include "dftg_internal.cuh"

namespace dftg {

constexpr int kKB = 32;   // points per shared-memory stage

template <typename T, int R, bool WJ>
__global__ void __launch_bounds__(256) k_contract(int nbf, int pts_per_chunk, size_t npad, const T *__restrict__ phi,
                                                  const T *__restrict__ cxc, const T *__restrict__ cj, int want_xc,
                                                  int want_j, const int2 *__restrict__ tiles,
                                                  double *__restrict__ part)
{
    constexpr int TILE = 16 * R;
    constexpr int LD = TILE + 1;
    __shared__ T sm_m[kKB * LD];
    __shared__ T sm_n[kKB * LD];
    __shared__ T sa[kKB], sb[kKB];
    const int2 tl = tiles[blockIdx.x];
    const int m0 = tl.x * TILE, n0 = tl.y * TILE;
    const int chunk = blockIdx.y;
    const size_t pb = (size_t)chunk * pts_per_chunk;
    const size_t pe = min(npad, pb + (size_t)pts_per_chunk);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    constexpr bool kF32 = sizeof(T) == 4;
    T ax[R][R], aj[R][R];
    // FP32: per-stage sums carried across stages as compensated (TwoSum) pairs
    float hx[R][R], lx[R][R], hj[R][R], lj[R][R];
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) {
            ax[i][j] = 0; aj[i][j] = 0;
            hx[i][j] = 0.f; lx[i][j] = 0.f; hj[i][j] = 0.f; lj[i][j] = 0.f;
        }

    for (size_t kb = pb; kb < pe; kb += kKB) {
        if constexpr (kF32) {
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int j = 0; j < R; ++j) { ax[i][j] = 0; aj[i][j] = 0; }
        }
        __syncthreads();
        for (int e = tid; e < TILE * kKB; e += 256) {
            const int row = e / kKB, k = e % kKB;
            const int mu = m0 + row, nu = n0 + row;
            sm_m[k * LD + row] = (mu < nbf) ? phi[(size_t)mu * npad + kb + k] : T(0);
            sm_n[k * LD + row] = (nu < nbf) ? phi[(size_t)nu * npad + kb + k] : T(0);
        }
        if (tid < kKB) {
            sa[tid] = want_xc ? cxc[kb + tid] : T(0);
            sb[tid] = want_j ? cj[kb + tid] : T(0);
        }
        __syncthreads();
#pragma unroll 4
        for (int k = 0; k < kKB; ++k) {
            T fm[R], fn[R];
#pragma unroll
            for (int i = 0; i < R; ++i) fm[i] = sm_m[k * LD + ty + 16 * i];
#pragma unroll
            for (int j = 0; j < R; ++j) fn[j] = sm_n[k * LD + tx + 16 * j];
            const T a = sa[k], b = sb[k];
#pragma unroll
            for (int i = 0; i < R; ++i) {
                const T u = a * fm[i], s = b * fm[i];
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    ax[i][j] += u * fn[j];
                    if constexpr (WJ) aj[i][j] += s * fn[j];
                }
            }
        }
        if constexpr (kF32) {
#pragma unroll
            for (int i = 0; i < R; ++i)
#pragma unroll
                for (int j = 0; j < R; ++j) {
                    two_sum_acc(hx[i][j], lx[i][j], (float)ax[i][j]);
                    if constexpr (WJ) two_sum_acc(hj[i][j], lj[i][j], (float)aj[i][j]);
                }
        }
    }
    const size_t nn = (size_t)nbf * nbf;
    double *px = part + (size_t)chunk * 2 * nn, *pj = px + nn;
#pragma unroll
    for (int i = 0; i < R; ++i)
#pragma unroll
        for (int j = 0; j < R; ++j) {
            const int mu = m0 + ty + 16 * i, nu = n0 + tx + 16 * j;
            if (mu < nbf && nu < nbf) {
                if constexpr (kF32) {
                    px[(size_t)mu * nbf + nu] = (double)hx[i][j] + (double)lx[i][j];
                    pj[(size_t)mu * nbf + nu] = (double)hj[i][j] + (double)lj[i][j];
                } else {
                    px[(size_t)mu * nbf + nu] = (double)ax[i][j];
                    pj[(size_t)mu * nbf + nu] = (double)aj[i][j];
                }
            }
        }
}

// sum partials of every computed element in chunk order; mirror below the
// diagonal blocks.  out matrices are column-major == row-major (symmetric).
// Block (32 elements x 8 chunk groups): group g sums chunks g, g+8, ... of its
// element (coalesced over the 32 elements), the 8 group sums are added in a
// fixed order, so the result does not depend on scheduling.
__global__ void __launch_bounds__(256) k_contract_reduce(int nbf, int tile, int nchunk, int want_xc, int want_j,
                                                         const double *__restrict__ part, double *__restrict__ XC,
                                                         double *__restrict__ J)
{
    __shared__ double shx[8][33], shj[8][33];
    const size_t nn = (size_t)nbf * nbf;
    const int lx = threadIdx.x & 31, g = threadIdx.x >> 5;
    const size_t e = (size_t)blockIdx.x * 32 + lx;
    double sx = 0.0, sj = 0.0;
    if (e < nn) {
        const int mu = (int)(e / nbf), nu = (int)(e % nbf);
        if (mu / tile <= nu / tile)
            for (int c = g; c < nchunk; c += 8) {
                const double *p = part + (size_t)c * 2 * nn;
                sx += p[e];
                sj += p[nn + e];
            }
    }
    shx[g][lx] = sx;
    shj[g][lx] = sj;
    __syncthreads();
    if (g != 0 || e >= nn) return;
    const int mu = (int)(e / nbf), nu = (int)(e % nbf);
    const int tm = mu / tile, tn = nu / tile;
    if (tm > tn) return;   // written by the mirror of (nu, mu)
    sx = shx[0][lx];
    sj = shj[0][lx];
    for (int k = 1; k < 8; ++k) {
        sx += shx[k][lx];
        sj += shj[k][lx];
    }
    // column-major element (row mu, col nu) sits at mu + nu*nbf
    if (want_xc) {
        XC[(size_t)nu * nbf + mu] = sx;
        if (tm < tn) XC[(size_t)mu * nbf + nu] = sx;
    }
    if (want_j) {
        J[(size_t)nu * nbf + mu] = sj;
        if (tm < tn) J[(size_t)mu * nbf + nu] = sj;
    }
}

// XC-only FP32 form for nbf > 128 (point sets, the dE/dP contraction of the
// backward pass): out = phi^T diag(coef) phi.  Output tiles of 128 (mu) x 64
// (nu) with block128(mu) <= block128(nu), split over point chunks like
// k_contract.  Per stage of 32 points, c o phi_mu (128 rows) and phi_nu (64 rows)
// are staged point-contiguous (row stride 36 floats: 16-byte rows, consecutive
// rows in distinct bank groups); thread (tx, ty) owns rows tx + 16 i (i < 8) and
// columns ty + 16 j (j < 4) and per four points loads 8 + 4 float4 for 128 FMAs.
// Stage sums are carried across stages as TwoSum pairs (as k_contract<float>).
constexpr int kXtM = 128, kXtN = 64, kXtK = 32, kXtLd = 36;

__host__ __device__ inline int xc32_tiles(int nbf)
{
    const int n128 = (nbf + kXtM - 1) / kXtM, n64 = (nbf + kXtN - 1) / kXtN;
    int t = 0;
    for (int mt = 0; mt < n128; ++mt) t += n64 - 2 * mt > 0 ? n64 - 2 * mt : 0;
    return t;
}

__device__ __forceinline__ void cp_async16(float *dst, const float *src)
{
    const unsigned d = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}

// one stage's panels: phi rows m0.. (A, scaled by coef after landing) and n0.. (B)
__device__ __forceinline__ void xc32_issue(float *As, float *Bs, int nbf, size_t npad, const float *phi, int m0, int n0,
                                           size_t kb, int tid)
{
    for (int e = tid; e < kXtM * (kXtK / 4); e += 256) {
        const int row = e >> 3, q = e & 7;
        float *d = As + row * kXtLd + 4 * q;
        if (m0 + row < nbf) cp_async16(d, phi + (size_t)(m0 + row) * npad + kb + 4 * q);
        else *reinterpret_cast<float4 *>(d) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    for (int e = tid; e < kXtN * (kXtK / 4); e += 256) {
        const int row = e >> 3, q = e & 7;
        float *d = Bs + row * kXtLd + 4 * q;
        if (n0 + row < nbf) cp_async16(d, phi + (size_t)(n0 + row) * npad + kb + 4 * q);
        else *reinterpret_cast<float4 *>(d) = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    asm volatile("cp.async.commit_group;" ::: "memory");
}

__global__ void __launch_bounds__(256) k_contract_xc32(int nbf, int pts_per_chunk, size_t npad,
                                                       const float *__restrict__ phi, const float *__restrict__ coef,
                                                       int slot, double *__restrict__ part)
{
    extern __shared__ __align__(16) float xsm[];   // two stages of As [128][36], Bs [64][36]
    const int n64 = (nbf + kXtN - 1) / kXtN;
    int t = blockIdx.x, mt = 0;
    while (t >= n64 - 2 * mt) { t -= n64 - 2 * mt; ++mt; }
    const int m0 = mt * kXtM, n0 = (2 * mt + t) * kXtN;
    const int chunk = blockIdx.y;
    const size_t pb = (size_t)chunk * pts_per_chunk;
    const size_t pe = min(npad, pb + (size_t)pts_per_chunk);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    constexpr int kStageF = (kXtM + kXtN) * kXtLd;
    float ax[8][4], hx[8][4], lx[8][4];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) { ax[i][j] = 0.f; hx[i][j] = 0.f; lx[i][j] = 0.f; }
    if (pb < pe) xc32_issue(xsm, xsm + kXtM * kXtLd, nbf, npad, phi, m0, n0, pb, tid);
    int buf = 0;
    for (size_t kb = pb; kb < pe; kb += kXtK, buf ^= 1) {
        float *As = xsm + buf * kStageF, *Bs = As + kXtM * kXtLd;
        if (kb + kXtK < pe) {
            float *An = xsm + (buf ^ 1) * kStageF;
            xc32_issue(An, An + kXtM * kXtLd, nbf, npad, phi, m0, n0, kb + kXtK, tid);
            asm volatile("cp.async.wait_group 1;" ::: "memory");
        } else {
            asm volatile("cp.async.wait_group 0;" ::: "memory");
        }
        __syncthreads();
        // c o phi_mu: row-wise scaling of the landed A panel
        for (int e = tid; e < kXtM * kXtK; e += 256) {
            const int row = e >> 5, k = e & 31;
            As[row * kXtLd + k] *= coef[kb + k];
        }
        __syncthreads();
#pragma unroll 2
        for (int k4 = 0; k4 < kXtK / 4; ++k4) {
            float4 a[8], b[4];
#pragma unroll
            for (int i = 0; i < 8; ++i) a[i] = *reinterpret_cast<const float4 *>(As + (tx + 16 * i) * kXtLd + 4 * k4);
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = *reinterpret_cast<const float4 *>(Bs + (ty + 16 * j) * kXtLd + 4 * k4);
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    ax[i][j] = fmaf(a[i].x, b[j].x, ax[i][j]);
                    ax[i][j] = fmaf(a[i].y, b[j].y, ax[i][j]);
                    ax[i][j] = fmaf(a[i].z, b[j].z, ax[i][j]);
                    ax[i][j] = fmaf(a[i].w, b[j].w, ax[i][j]);
                }
        }
#pragma unroll
        for (int i = 0; i < 8; ++i)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                two_sum_acc(hx[i][j], lx[i][j], ax[i][j]);
                ax[i][j] = 0.f;
            }
        __syncthreads();   // this buffer is refilled by the prefetch of the next iteration
    }
    double *px = part + ((size_t)chunk * 2 + slot) * nbf * nbf;   // slot 0: XC, 1: J
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int mu = m0 + tx + 16 * i, nu = n0 + ty + 16 * j;
            if (mu < nbf && nu < nbf) px[(size_t)mu * nbf + nu] = (double)hx[i][j] + (double)lx[i][j];
        }
}

constexpr size_t kXtSmem = 2 * (size_t)(kXtM + kXtN) * kXtLd * sizeof(float);

static int tile_R(int nbf) { return nbf <= 80 ? 5 : 4; }

size_t contract_part_elems(int nbf, size_t npad)
{
    const int R = tile_R(nbf), tile = 16 * R;
    const int nt = (nbf + tile - 1) / tile;
    const int npairs = nt * (nt + 1) / 2;
    int nchunk = (2 * 152 + npairs - 1) / npairs;
    if (nbf > 128) nchunk = max(nchunk, (4 * 152 + xc32_tiles(nbf) - 1) / xc32_tiles(nbf));
    const size_t max_chunks = npad / (4 * kKB);
    if ((size_t)nchunk > max_chunks) nchunk = (int)(max_chunks > 0 ? max_chunks : 1);
    return (size_t)nchunk * 2 * nbf * nbf;
}

int contract_setup(dftg_ctx *c)
{
    const int R = tile_R(c->nbf), tile = 16 * R;
    const int nt = (c->nbf + tile - 1) / tile;
    std::vector<int2> tl;
    for (int a = 0; a < nt; ++a)
        for (int b = a; b < nt; ++b) tl.push_back(make_int2(a, b));
    c->ntiles = (int)tl.size();
    c->nchunk = (int)(contract_part_elems(c->nbf, c->npad) / (2 * (size_t)c->nbf * c->nbf));
    DFTG_CUDA(cudaMalloc(&c->d_tiles, sizeof(int2) * tl.size()));
    DFTG_CUDA(cudaMemcpy(c->d_tiles, tl.data(), sizeof(int2) * tl.size(), cudaMemcpyHostToDevice));
    return DFTG_OK;
}

// k_contract with the J accumulators only when J is wanted
template <typename T, int R>
static void contract_launch(dim3 grid, cudaStream_t st, int nbf, int per, size_t npad, const T *phi, const T *cxc,
                            const T *cj, int wx, int wj, const int2 *tiles, double *part)
{
    if (wj) k_contract<T, R, true><<<grid, 256, 0, st>>>(nbf, per, npad, phi, cxc, cj, wx, wj, tiles, part);
    else k_contract<T, R, false><<<grid, 256, 0, st>>>(nbf, per, npad, phi, cxc, cj, wx, wj, tiles, part);
}

int launch_contract(dftg_ctx *c, bool want_xc, bool want_j)
{
    const int wx = want_xc ? 1 : 0, wj = want_j ? 1 : 0;
    const size_t nn = (size_t)c->nbf * c->nbf;
    if ((c->prec_mask & kPrecContract) && c->ct_ready) {
        // tensor-core form: full nbf x nbf partials per CTA, upper triangle kept
        DFTG_TRY_L(launch_contract_tc(c));
        DFTG_MARK(c, "contract");
        DFTG_TRY_L(launch_contract_tc_reduce(c, want_xc, want_j));
        DFTG_MARK(c, "contract_reduce");
        return DFTG_OK;
    }
    const int R = tile_R(c->nbf), tile = 16 * R;
    const int2 *d_tiles = reinterpret_cast<const int2 *>(c->d_tiles);
    size_t per = (c->npad + c->nchunk - 1) / c->nchunk;
    per = (per + kKB - 1) / kKB * kKB;
    dim3 grid((unsigned)c->ntiles, (unsigned)c->nchunk);
    if (!(c->prec_mask & kPrecContract)) {
        if (R == 5) contract_launch<double, 5>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi, c->d_cxc, c->d_cj, wx, wj, d_tiles, c->d_part);
        else contract_launch<double, 4>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi, c->d_cxc, c->d_cj, wx, wj, d_tiles, c->d_part);
    } else if (c->nbf > 128 && c->tt_ready) {
        // tensor-core tiles, one pass per wanted matrix
        DFTG_TRY_L(launch_contract_tt_bounds(c, c->d_cxc32, c->d_cj32));
        DFTG_MARK(c, "contract_bounds");
        if (want_xc) DFTG_TRY_L(launch_contract_tt(c, c->d_cxc32, 0, c->d_XC));
        if (want_j) DFTG_TRY_L(launch_contract_tt(c, c->d_cj32, 1, c->d_J));
        return DFTG_OK;
    } else if (c->nbf > 128) {
        // one tiled pass per wanted matrix (the J pass reads the amplitudes again)
        const dim3 g2((unsigned)xc32_tiles(c->nbf), (unsigned)c->nchunk);
        DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_contract_xc32), c->device));
        if (want_xc)
            k_contract_xc32<<<g2, 256, kXtSmem, c->stream>>>(c->nbf, (int)per, c->npad, c->d_phi32, c->d_cxc32, 0,
                                                            c->d_part);
        if (want_j)
            k_contract_xc32<<<g2, 256, kXtSmem, c->stream>>>(c->nbf, (int)per, c->npad, c->d_phi32, c->d_cj32, 1,
                                                            c->d_part);
        DFTG_LAUNCH_CHECK();
        DFTG_MARK(c, "contract");
        k_contract_reduce<<<(unsigned)((nn + 31) / 32), 256, 0, c->stream>>>(c->nbf, kXtM, c->nchunk, wx, wj, c->d_part,
                                                                             c->d_XC, c->d_J);
        DFTG_LAUNCH_CHECK();
        DFTG_MARK(c, "contract_reduce");
        return DFTG_OK;
    } else {
        if (R == 5) contract_launch<float, 5>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi32, c->d_cxc32, c->d_cj32, wx, wj, d_tiles, c->d_part);
        else contract_launch<float, 4>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi32, c->d_cxc32, c->d_cj32, wx, wj, d_tiles, c->d_part);
    }
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "contract");
    k_contract_reduce<<<(unsigned)((nn + 31) / 32), 256, 0, c->stream>>>(c->nbf, tile, c->nchunk, wx, wj, c->d_part,
                                                                        c->d_XC, c->d_J);
    DFTG_LAUNCH_CHECK();
    DFTG_MARK(c, "contract_reduce");
    return DFTG_OK;
}

// out = phi^T diag(coef) phi in FP64 (the same kernels as the FP64 XC step),
// for contractions with other point weights (the backward pass)
int launch_contract_coef(dftg_ctx *c, const double *coef, double *out)
{
    const int R = tile_R(c->nbf), tile = 16 * R;
    const int2 *d_tiles = reinterpret_cast<const int2 *>(c->d_tiles);
    size_t per = (c->npad + c->nchunk - 1) / c->nchunk;
    per = (per + kKB - 1) / kKB * kKB;
    dim3 grid((unsigned)c->ntiles, (unsigned)c->nchunk);
    if (R == 5) contract_launch<double, 5>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi, coef, coef, 1, 0, d_tiles, c->d_part);
    else contract_launch<double, 4>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi, coef, coef, 1, 0, d_tiles, c->d_part);
    DFTG_LAUNCH_CHECK();
    const size_t nn = (size_t)c->nbf * c->nbf;
    k_contract_reduce<<<(unsigned)((nn + 31) / 32), 256, 0, c->stream>>>(c->nbf, tile, c->nchunk, 1, 0, c->d_part,
                                                                        out, nullptr);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// the same in FP32 (products and in-chunk sums; FP64 across chunks) from the FP32 amplitudes
int launch_contract_coef32(dftg_ctx *c, const float *coef, double *out)
{
    const int R = tile_R(c->nbf), tile = 16 * R;
    const int2 *d_tiles = reinterpret_cast<const int2 *>(c->d_tiles);
    size_t per = (c->npad + c->nchunk - 1) / c->nchunk;
    per = (per + kKB - 1) / kKB * kKB;
    dim3 grid((unsigned)c->ntiles, (unsigned)c->nchunk);
    int rtile = tile;
    if (c->nbf > 128 && c->tt_ready) {
        DFTG_TRY_L(launch_contract_tt_bounds(c, coef, coef));
        return launch_contract_tt(c, coef, 0, out);
    }
    if (c->nbf > 128) {
        const dim3 g2((unsigned)xc32_tiles(c->nbf), (unsigned)c->nchunk);
        DFTG_TRY_L(allow_max_dyn_smem(reinterpret_cast<const void *>(k_contract_xc32), c->device));
        k_contract_xc32<<<g2, 256, kXtSmem, c->stream>>>(c->nbf, (int)per, c->npad, c->d_phi32, coef, 0, c->d_part);
        rtile = kXtM;
    } else if (R == 5) {
        contract_launch<float, 5>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi32, coef, coef, 1, 0, d_tiles, c->d_part);
    } else {
        contract_launch<float, 4>(grid, c->stream, c->nbf, (int)per, c->npad, c->d_phi32, coef, coef, 1, 0, d_tiles, c->d_part);
    }
    DFTG_LAUNCH_CHECK();
    const size_t nn = (size_t)c->nbf * c->nbf;
    k_contract_reduce<<<(unsigned)((nn + 31) / 32), 256, 0, c->stream>>>(c->nbf, rtile, c->nchunk, 1, 0, c->d_part,
                                                                        out, nullptr);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

}  // namespace dftg
