// k_contract_noalloc.cu -- the XC/J contraction without any device allocation.
//
// Some callers cannot allocate device memory: a host program whose framework
// owns every byte of GPU memory (one pool or arena reserved at start-up), or a
// service that runs under a fixed device-memory budget, may not call
// cudaMalloc / cudaFree (or any allocating library routine) while it serves
// requests.  dftg_contract_noalloc serves them: it computes
//   XC = phi^T diag(cxc) phi   and   J = phi^T diag(cj) phi
// from caller-owned device buffers and keeps its split-K partial sums in the
// file-scope array below, which is part of the library image: every GPU that
// loads the library holds DFTG_NOALLOC_SCRATCH_BYTES of device memory for it
// until the process exits.
//
// Set-up: every call looks up the array's device address on the current
// device with cudaGetSymbolAddress (a host-side lookup that allocates nothing),
// so the address stays right when the device's context is torn down and made
// again.  The first call on a device also loads the library's device code
// there; make it before any stream capture.  Calls share the array: two calls
// that overlap on the GPU (different streams, or different host threads) race.
// Every partial sum a call reads is written earlier by the same call, so no
// part of the array needs clearing between calls.
#include "dftg_internal.cuh"

namespace dftg {

constexpr size_t kNoallocScratchDoubles = DFTG_NOALLOC_SCRATCH_BYTES / sizeof(double);
static __device__ __align__(256) double g_noalloc_scratch[kNoallocScratchDoubles];

constexpr int kNaR = 4, kNaTile = 16 * kNaR, kNaKB = 32;

// upper-triangular block index -> (row block, column block)
__device__ __forceinline__ void tile_of(int t, int nt, int &a, int &b)
{
    a = 0;
    while (t >= nt - a) { t -= nt - a; ++a; }
    b = a + t;
}

__global__ void __launch_bounds__(256) k_contract_na(int nbf, size_t npts, size_t ld, int pts_per_chunk,
                                                     const double *__restrict__ phi, const double *__restrict__ cxc,
                                                     const double *__restrict__ cj, double *__restrict__ part)
{
    constexpr int LD = kNaTile + 1;
    __shared__ double sm_m[kNaKB * LD];
    __shared__ double sm_n[kNaKB * LD];
    __shared__ double sa[kNaKB], sb[kNaKB];
    const int nt = (nbf + kNaTile - 1) / kNaTile;
    int ta, tb;
    tile_of(blockIdx.x, nt, ta, tb);
    const int m0 = ta * kNaTile, n0 = tb * kNaTile;
    const int chunk = blockIdx.y;
    const size_t pb = (size_t)chunk * pts_per_chunk;
    const size_t pe = min(npts, pb + (size_t)pts_per_chunk);
    const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
    double ax[kNaR][kNaR], aj[kNaR][kNaR];
#pragma unroll
    for (int i = 0; i < kNaR; ++i)
#pragma unroll
        for (int j = 0; j < kNaR; ++j) { ax[i][j] = 0.0; aj[i][j] = 0.0; }
    for (size_t kb = pb; kb < pe; kb += kNaKB) {
        __syncthreads();
        for (int e = tid; e < kNaTile * kNaKB; e += 256) {
            const int row = e / kNaKB, k = e % kNaKB;
            const size_t p = kb + k;
            const int mu = m0 + row, nu = n0 + row;
            sm_m[k * LD + row] = (mu < nbf && p < pe) ? phi[(size_t)mu * ld + p] : 0.0;
            sm_n[k * LD + row] = (nu < nbf && p < pe) ? phi[(size_t)nu * ld + p] : 0.0;
        }
        if (tid < kNaKB) {
            const size_t p = kb + tid;
            sa[tid] = p < pe ? cxc[p] : 0.0;
            sb[tid] = p < pe ? cj[p] : 0.0;
        }
        __syncthreads();
        for (int k = 0; k < kNaKB; ++k) {
            double fm[kNaR], fn[kNaR];
#pragma unroll
            for (int i = 0; i < kNaR; ++i) fm[i] = sm_m[k * LD + ty + 16 * i];
#pragma unroll
            for (int j = 0; j < kNaR; ++j) fn[j] = sm_n[k * LD + tx + 16 * j];
            const double a = sa[k], b = sb[k];
#pragma unroll
            for (int i = 0; i < kNaR; ++i) {
                const double u = a * fm[i], s = b * fm[i];
#pragma unroll
                for (int j = 0; j < kNaR; ++j) {
                    ax[i][j] += u * fn[j];
                    aj[i][j] += s * fn[j];
                }
            }
        }
    }
    const size_t nn = (size_t)nbf * nbf;
    double *px = part + (size_t)chunk * 2 * nn, *pj = px + nn;
#pragma unroll
    for (int i = 0; i < kNaR; ++i)
#pragma unroll
        for (int j = 0; j < kNaR; ++j) {
            const int mu = m0 + ty + 16 * i, nu = n0 + tx + 16 * j;
            if (mu < nbf && nu < nbf) {
                px[(size_t)mu * nbf + nu] = ax[i][j];
                pj[(size_t)mu * nbf + nu] = aj[i][j];
            }
        }
}

__global__ void k_contract_na_reduce(int nbf, int nchunk, const double *__restrict__ part, double *__restrict__ XC,
                                     double *__restrict__ J)
{
    const size_t nn = (size_t)nbf * nbf;
    const size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= nn) return;
    const int mu = (int)(e / nbf), nu = (int)(e % nbf);
    const int tm = mu / kNaTile, tn = nu / kNaTile;
    if (tm > tn) return;
    double sx = 0.0, sj = 0.0;
    for (int c = 0; c < nchunk; ++c) {
        sx += part[(size_t)c * 2 * nn + e];
        sj += part[(size_t)c * 2 * nn + nn + e];
    }
    if (XC) {
        XC[(size_t)nu * nbf + mu] = sx;
        if (tm < tn) XC[(size_t)mu * nbf + nu] = sx;
    }
    if (J) {
        J[(size_t)nu * nbf + mu] = sj;
        if (tm < tn) J[(size_t)mu * nbf + nu] = sj;
    }
}

// device address of the scratch array on the current device
static int noalloc_scratch(double **out)
{
    void *p = nullptr;
    DFTG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    *out = static_cast<double *>(p);
    return DFTG_OK;
}

}  // namespace dftg

extern "C" int dftg_contract_noalloc(const double *phi, size_t ld, size_t npts, int nbf, const double *cxc,
                                     const double *cj, double *XC, double *J, void *stream)
{
    using namespace dftg;
    if (!phi || !cxc || !cj || (!XC && !J)) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    if (nbf < 1 || npts < 1 || ld < npts) { set_error("bad sizes: nbf %d npts %zu ld %zu", nbf, npts, ld); return DFTG_ERR_ARG; }
    const size_t per_chunk = 2 * (size_t)nbf * nbf;
    if (per_chunk > kNoallocScratchDoubles) {
        set_error("nbf %d exceeds the no-allocation limit %d (scratch %zu bytes)", nbf, DFTG_NOALLOC_MAX_NBF,
                  (size_t)DFTG_NOALLOC_SCRATCH_BYTES);
        return DFTG_ERR_ARG;
    }
    double *scratch = nullptr;
    int rc = noalloc_scratch(&scratch);
    if (rc != DFTG_OK) return rc;
    const int nt = (nbf + kNaTile - 1) / kNaTile;
    const int ntiles = nt * (nt + 1) / 2;
    size_t nchunk = (2 * 152 + ntiles - 1) / ntiles;
    const size_t fit = kNoallocScratchDoubles / per_chunk;
    if (nchunk > fit) nchunk = fit;
    const size_t max_chunks = (npts + 4 * kNaKB - 1) / (4 * kNaKB);
    if (nchunk > max_chunks) nchunk = max_chunks;
    if (nchunk < 1) nchunk = 1;
    size_t per = (npts + nchunk - 1) / nchunk;
    per = (per + kNaKB - 1) / kNaKB * kNaKB;
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    dim3 grid((unsigned)ntiles, (unsigned)nchunk);
    k_contract_na<<<grid, 256, 0, s>>>(nbf, npts, ld, (int)per, phi, cxc, cj, scratch);
    DFTG_CUDA(cudaGetLastError());
    const size_t nn = (size_t)nbf * nbf;
    k_contract_na_reduce<<<(unsigned)((nn + 255) / 256), 256, 0, s>>>(nbf, (int)nchunk, scratch, XC, J);
    DFTG_CUDA(cudaGetLastError());
    return DFTG_OK;
}
