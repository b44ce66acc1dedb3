// k_scf.cu -- device SCF driver: the reference's DFT constructor and DFT::scf
// (dft.cpp:57-61, 84-142, 160-227, 300-366, 441-447) with every step on the GPU,
// and the whole loop as one CUDA graph launch.
//
// Eigen-solver.  FP64 arithmetic on this GPU runs at a small fraction of the
// FP32 rate, so an O(n^3) FP64 eigen-solve inside one CTA would take
// milliseconds.  It is split in two:
//   1. cyclic Jacobi rotations in FP32 in one CTA of 1024 threads, A and the
//      accumulated rotations V in shared memory (n <= 160).  A step applies
//      n/2 disjoint rotations chosen by the round-robin (circle) ordering as
//      2 x 2 block updates G_u^T A_uw G_w, two barriers per step;
//   2. FP64 iterative refinement of the eigenvectors after Ogita and Aishima,
//      "Iterative refinement for symmetric eigenvalue decomposition", Japan J.
//      Indust. Appl. Math. 35 (2018) 1007-1035.  With G = V^T V, S = V^T A V,
//      lambda_i = s_ii / g_ii and R = I - G, V <- V (I + E) where
//        e_ij = (s_ij + lambda_j r_ij) / (lambda_j - lambda_i)   i and j on
//               different sides of the occupied / virtual split,
//        e_ij = r_ij / 2                                          same side.
//      Only the occupied subspace enters P, so vectors on the same side are
//      re-orthonormalised and pairs across the split converge quadratically.
//      A cross pair with a gap below 1e-12 ||A||_F (a degenerate HOMO / LUMO,
//      where the split is arbitrary in any solver) or a first-order correction
//      above 1 is treated as a same-side pair.  The GEMMs run in FP64 on many
//      CTAs (8 x 8 output tiles).
// X = U diag(lambda^-1/2) from the FP32 eigenpairs of S, then Newton-Schulz
// steps X <- X (3I - X^T S X) / 2 until X^T S X = I to FP64 accuracy.  P does
// not depend on which X is used as long as X^T S X = I.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstring>
#include "dftg_internal.cuh"

namespace dftg {
namespace {

constexpr int kScfMaxN = DFTG_SCF_MAX_NBF;
constexpr int kJacobiThreads = 1024;
constexpr int kJacobiMaxSweeps = 30;
constexpr float kJacobiTol = 2e-7f;      // rotation threshold, relative to ||A||_F
constexpr int kNsSteps = 4;              // Newton-Schulz steps for X^T S X = I
constexpr int kRefineDefault = 4;
constexpr double kDegenerateRel = 1e-12; // cross pairs closer than this (x ||A||_F) are not split
constexpr int kHistW = DFTG_SCF_HIST_W;

// slots of the device state vector
enum {
    kStE = 0,       // energy of the last iteration (E_0 after set-up)
    kStIt = 1,      // iterations of the current run
    kStDiff = 2,    // |E_n - E_(n-1)|
    kStCont = 3,    // 1: the loop continues
    kStAnorm = 4,   // ||A||_F of the last eigen-solve
    kStSweeps = 5,  // Jacobi sweeps of the last eigen-solve
    kStCross = 6,   // max |s_ij| across the split, last refinement step
    kStOrth = 7,    // max |r_ij|, last refinement step
    kStLamMin = 8,  // smallest Jacobi eigenvalue (positive definiteness of S)
    kStElems = 16
};

// ------------------------------------------------------------------ kernels

// Cyclic Jacobi in FP32 (one CTA): A (n x n, column-major, symmetric) -> V
// (columns: eigenvectors, FP64 storage of the FP32 values), lam (diagonal).
// A step rotates the pairs of one round of the circle ordering whose
// off-diagonal element exceeds the threshold; only their 2 x 2 blocks of A and
// their columns of V are touched (a warp per rotated pair, lanes along the
// other index), so late sweeps with few rotations cost little.  The list of
// rotated pairs is built with a shared counter; its order does not change any
// value, since every block update depends on its two pairs only.
__global__ void __launch_bounds__(kJacobiThreads) k_scf_jacobi(int n, const double *__restrict__ A,
                                                               double *__restrict__ V, double *__restrict__ lam,
                                                               double *__restrict__ st)
{
    extern __shared__ float sm[];
    __shared__ double s_red[32];
    __shared__ int s_rot, s_nrot[2];
    __shared__ int s_list[kScfMaxN / 2];
    const int np = n + (n & 1), ld = np + 1, h = np / 2, m = np - 1;
    const int tid = threadIdx.x, nt = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nt >> 5;
    float *a = sm;
    float *v = a + np * ld;
    float2 *cs = reinterpret_cast<float2 *>(v + np * ld);   // np * ld is even: 8-byte aligned
    int2 *pq = reinterpret_cast<int2 *>(cs + h);

    double nrm = 0.0;
    for (int j = warp; j < np; j += nwarps)
        for (int i = lane; i < np; i += 32) {
            const double x = (i < n && j < n) ? A[i + (size_t)j * n] : 0.0;
            nrm += x * x;
            a[i * ld + j] = (float)x;
            v[i * ld + j] = (i == j) ? 1.f : 0.f;
        }
    nrm = block_sum(nrm, s_red);
    if (tid == 0) {
        s_red[0] = nrm;
        s_nrot[0] = 0;
        s_nrot[1] = 0;
    }
    __syncthreads();
    const double anorm = sqrt(s_red[0]);
    const float tol = kJacobiTol * (float)anorm;

    int sweep = 0, step = 0;
    for (; sweep < kJacobiMaxSweeps; ++sweep) {
        if (tid == 0) s_rot = 0;
        __syncthreads();
        for (int k = 0; k < m; ++k, ++step) {
            const int cur = step & 1;
            if (tid < h) {
                int p = (tid == 0) ? k : (k + tid) % m;
                int q = (tid == 0) ? m : (k - tid + m) % m;
                if (p > q) { const int t = p; p = q; q = t; }
                const float apq = a[p * ld + q];
                float c = 1.f, s = 0.f;
                if (fabsf(apq) > tol) {
                    const float app = a[p * ld + p], aqq = a[q * ld + q];
                    const float th = (aqq - app) / (2.f * apq);
                    const float t = copysignf(1.f, th) / (fabsf(th) + sqrtf(fmaf(th, th, 1.f)));
                    c = 1.f / sqrtf(fmaf(t, t, 1.f));
                    s = t * c;
                    s_list[atomicAdd(&s_nrot[cur], 1)] = tid;
                    s_rot = 1;
                }
                cs[tid] = make_float2(c, s);
                pq[tid] = make_int2(p, q);
            }
            __syncthreads();
            const int nrot = s_nrot[cur];
            if (tid == 0) s_nrot[cur ^ 1] = 0;   // counter of the next step (read by nobody now)
            for (int e = warp; e < nrot; e += nwarps) {
                const int u = s_list[e];
                const float2 gu = cs[u];
                const int2 iu = pq[u];
                // A <- G^T A G on the blocks (u, w); a block of two rotated pairs is
                // done once, by the smaller pair index; mirrored below the diagonal
                for (int w = lane; w < h; w += 32) {
                    const float2 gw = cs[w];
                    if (gw.y != 0.f && w < u) continue;
                    const int2 iw = pq[w];
                    const float xpp = a[iu.x * ld + iw.x], xpq = a[iu.x * ld + iw.y];
                    const float xqp = a[iu.y * ld + iw.x], xqq = a[iu.y * ld + iw.y];
                    const float ypp = gw.x * xpp - gw.y * xpq, ypq = gw.y * xpp + gw.x * xpq;
                    const float yqp = gw.x * xqp - gw.y * xqq, yqq = gw.y * xqp + gw.x * xqq;
                    const float zpp = gu.x * ypp - gu.y * yqp, zqp = gu.y * ypp + gu.x * yqp;
                    const float zpq = gu.x * ypq - gu.y * yqq, zqq = gu.y * ypq + gu.x * yqq;
                    if (w == u) {
                        a[iu.x * ld + iu.x] = zpp;
                        a[iu.y * ld + iu.y] = zqq;
                        a[iu.x * ld + iu.y] = 0.f;
                        a[iu.y * ld + iu.x] = 0.f;
                    } else {
                        a[iu.x * ld + iw.x] = zpp; a[iu.x * ld + iw.y] = zpq;
                        a[iu.y * ld + iw.x] = zqp; a[iu.y * ld + iw.y] = zqq;
                        a[iw.x * ld + iu.x] = zpp; a[iw.y * ld + iu.x] = zpq;
                        a[iw.x * ld + iu.y] = zqp; a[iw.y * ld + iu.y] = zqq;
                    }
                }
                // V <- V G on the two columns of pair u
                for (int r = lane; r < np; r += 32) {
                    const float vp = v[r * ld + iu.x], vq = v[r * ld + iu.y];
                    v[r * ld + iu.x] = gu.x * vp - gu.y * vq;
                    v[r * ld + iu.y] = gu.y * vp + gu.x * vq;
                }
            }
            __syncthreads();
        }
        const int rot = s_rot;
        __syncthreads();
        if (!rot) break;
    }
    for (int col = warp; col < n; col += nwarps)
        for (int r = lane; r < n; r += 32) V[r + (size_t)col * n] = (double)v[r * ld + col];
    for (int i = tid; i < n; i += nt) lam[i] = (double)a[i * ld + i];
    if (tid == 0) {
        float mn = a[0];
        for (int i = 1; i < n; ++i) mn = fminf(mn, a[i * ld + i]);
        st[kStAnorm] = anorm;
        st[kStSweeps] = (double)(sweep < kJacobiMaxSweeps ? sweep + 1 : sweep);
        st[kStLamMin] = (double)mn;
    }
}

size_t jacobi_smem(int n)
{
    const int np = n + (n & 1);
    return sizeof(float) * 2 * (size_t)np * (np + 1) + (sizeof(float2) + sizeof(int2)) * (size_t)(np / 2);
}

// C = alpha op(A) op(B)[:, bcol] + beta C0 in FP64; op = transpose when t* set.
// C0 may equal C (each element is read and written by one thread); A and B
// must not overlap C.
struct GemmOp {
    int m, n, k, ta, tb, lda, ldb, ldc;
    double alpha, beta;
    const double *A, *B, *C0;
    const int *bcol;
    double *C;
};

// 8 x 8 output tile per CTA of 64 threads; K in panels of 64 staged in shared
// memory with coalesced loads (the operands live in L2), then a sequential FMA
// chain per output element in increasing K.
constexpr int kGT = 8, kGK = 64;
__global__ void __launch_bounds__(64) k_scf_gemm(GemmOp g0, GemmOp g1)
{
    __shared__ double As[kGK][kGT + 1];   // As[l][r] = op(A)(i0 + r, l0 + l)
    __shared__ double Bs[kGK][kGT + 1];   // Bs[l][c] = op(B)(l0 + l, j0 + c)
    const GemmOp g = blockIdx.z ? g1 : g0;
    const int i0 = blockIdx.x * kGT, j0 = blockIdx.y * kGT;
    if (i0 >= g.m || j0 >= g.n) return;   // uniform over the CTA
    const int ii = threadIdx.x & 7, jj = threadIdx.x >> 3;
    double s = 0.0;
    for (int l0 = 0; l0 < g.k; l0 += kGK) {
        const int kc = min(kGK, g.k - l0);
        for (int e = threadIdx.x; e < kGT * kGK; e += 64) {
            int r, l;   // A element: contiguous along i when not transposed, along l when transposed
            if (!g.ta) { r = e & 7; l = e >> 3; } else { l = e % kGK; r = e / kGK; }
            double v = 0.0;
            if (l < kc && i0 + r < g.m)
                v = g.ta ? g.A[(l0 + l) + (size_t)(i0 + r) * g.lda] : g.A[(i0 + r) + (size_t)(l0 + l) * g.lda];
            As[l][r] = v;
            int cb, lb;  // B element: contiguous along l when not transposed, along j when transposed
            if (!g.tb) { lb = e % kGK; cb = e / kGK; } else { cb = e & 7; lb = e >> 3; }
            double w = 0.0;
            if (lb < kc && j0 + cb < g.n) {
                const int jb = g.bcol ? g.bcol[j0 + cb] : j0 + cb;
                w = g.tb ? g.B[jb + (size_t)(l0 + lb) * g.ldb] : g.B[(l0 + lb) + (size_t)jb * g.ldb];
            }
            Bs[lb][cb] = w;
        }
        __syncthreads();
        for (int l = 0; l < kc; ++l) s = fma(As[l][ii], Bs[l][jj], s);
        __syncthreads();
    }
    const int i = i0 + ii, j = j0 + jj;
    if (i >= g.m || j >= g.n) return;
    double r = g.alpha * s;
    if (g.beta != 0.0) r += g.beta * g.C0[i + (size_t)j * g.ldc];
    g.C[i + (size_t)j * g.ldc] = r;
}

// out = a X + b Y + c Z (n2 elements; Y or Z may be NULL)
__global__ void k_scf_axpby(int n2, double a, const double *__restrict__ X, double b, const double *__restrict__ Y,
                            double c, const double *__restrict__ Z, double *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n2) return;
    double r = a * X[i];
    if (Y) r += b * Y[i];
    if (Z) r += c * Z[i];
    out[i] = r;
}

// X = U diag(lam^-1/2)
__global__ void k_scf_scale_cols(int n, const double *__restrict__ U, const double *__restrict__ lam,
                                 double *__restrict__ X)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n * n) return;
    X[i] = U[i] / sqrt(lam[i / n]);
}

__device__ __forceinline__ double block_max(double v, double *sh)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s = fmax(s, sh[i]);
    __syncthreads();
    return s;
}

// integer key with the order of the doubles (negative values: magnitude bits flipped)
__device__ __forceinline__ long long order_key(double x)
{
    const long long b = __double_as_longlong(x);
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

// One refinement step: E from G = V^T V and S = V^T A V over a grid of CTAs
// (256 elements each).  Every CTA forms the eigenvalue estimates and their
// ranks (integer keys, ties by index); CTA 0 writes the ascending estimates
// (eps) and the permutation that sorts them.  The residual maxima go to the
// state vector by atomicMax on the bits of non-negative doubles (zeroed before
// the launch), so their value does not depend on the CTA order.
__global__ void __launch_bounds__(256) k_scf_refine(int n, int nocc, const double *__restrict__ G,
                                                    const double *__restrict__ S, double *__restrict__ E,
                                                    double *__restrict__ eps, int *__restrict__ perm,
                                                    double *__restrict__ st)
{
    __shared__ double s_lam[kScfMaxN];
    __shared__ long long s_key[kScfMaxN];
    __shared__ int s_occ[kScfMaxN];
    __shared__ double s_red[32];
    const int tid = threadIdx.x, nt = blockDim.x;
    for (int i = tid; i < n; i += nt) {
        const double l = S[i + (size_t)i * n] / G[i + (size_t)i * n];
        s_lam[i] = l;
        s_key[i] = order_key(l);
    }
    __syncthreads();
    for (int i = tid; i < n; i += nt) {
        const long long ki = s_key[i];
        int rank = 0;
        for (int j = 0; j < n; ++j) {
            const long long kj = s_key[j];
            rank += (kj < ki || (kj == ki && j < i)) ? 1 : 0;
        }
        s_occ[i] = rank < nocc;
        if (blockIdx.x == 0) {
            perm[rank] = i;
            eps[rank] = s_lam[i];
        }
    }
    __syncthreads();
    const double tau = kDegenerateRel * st[kStAnorm];
    double cmax = 0.0, rmax = 0.0;
    const int idx = blockIdx.x * nt + tid;
    if (idx < n * n) {
        const int i = idx % n, j = idx / n;
        const double r = (i == j ? 1.0 : 0.0) - G[idx];
        double e = 0.5 * r;
        if (s_occ[i] != s_occ[j]) {
            const double den = s_lam[j] - s_lam[i];
            const double num = S[idx] + s_lam[j] * r;
            if (fabs(den) > tau && fabs(num) < fabs(den)) e = num / den;
            cmax = fabs(S[idx]);
        }
        rmax = fabs(r);
        E[idx] = e;
    }
    cmax = block_max(cmax, s_red);
    rmax = block_max(rmax, s_red);
    if (tid == 0) {
        atomicMax(reinterpret_cast<unsigned long long *>(st + kStCross), (unsigned long long)__double_as_longlong(cmax));
        atomicMax(reinterpret_cast<unsigned long long *>(st + kStOrth), (unsigned long long)__double_as_longlong(rmax));
    }
}

// Energy (dft.cpp:441-447) and the loop test of DFT::scf (dft.cpp:95-131).
// init: E_0 of the set-up (E_xc = 0, E_J = 2 tr(P J)), no iteration counted.
__global__ void __launch_bounds__(256) k_scf_energy(int n, const double *__restrict__ P, const double *__restrict__ H,
                                                    const double *__restrict__ J, const double *__restrict__ scal,
                                                    int init, int grid_ej, double enuc, double tol, int min_iter,
                                                    int max_iter, double *__restrict__ st, double *__restrict__ hist,
                                                    cudaGraphConditionalHandle handle, int has_cond)
{
    __shared__ double s_red[32];
    double ph = 0.0, pj = 0.0;
    for (int i = threadIdx.x; i < n * n; i += blockDim.x) {
        ph += P[i] * H[i];
        pj += P[i] * J[i];
    }
    ph = block_sum(ph, s_red);
    pj = block_sum(pj, s_red);
    if (threadIdx.x != 0) return;
    const double e1 = 2.0 * ph;
    const double ej = (grid_ej && !init) ? scal[kScalEJ] : 2.0 * pj;
    const double exc = init ? 0.0 : scal[kScalExc];
    const double E = e1 + ej + enuc + exc;
    if (init) {
        st[kStE] = E;
        st[kStIt] = 0.0;
        st[kStDiff] = 1.0;
        st[kStCont] = 1.0;
        return;
    }
    const int it = (int)st[kStIt] + 1;
    const double diff = fabs(E - st[kStE]);
    st[kStE] = E;
    st[kStIt] = (double)it;
    st[kStDiff] = diff;
    if (it - 1 < max_iter) {
        double *row = hist + (size_t)(it - 1) * kHistW;
        row[0] = E;
        row[1] = e1;
        row[2] = ej;
        row[3] = exc;
        row[4] = scal[kScalNelec];
        row[5] = diff;
    }
    const bool cont = (diff > tol || it < min_iter) && it < max_iter;
    st[kStCont] = cont ? 1.0 : 0.0;
    if (has_cond) cudaGraphSetConditional(handle, cont ? 1u : 0u);
}

}  // namespace
}  // namespace dftg

struct dftg_scf_state {
    int n = 0, nocc = 0, nref = 4, min_iter = 3, max_iter = 100;
    double alpha = 0.5, tol = 1e-4, enuc = 0.0;
    double *buf = nullptr;
    double *H = nullptr, *X = nullptr, *X2 = nullptr, *F = nullptr, *T = nullptr, *Fp = nullptr, *V0 = nullptr,
           *V1 = nullptr, *Vk = nullptr, *G = nullptr, *W = nullptr, *S = nullptr, *E = nullptr, *C = nullptr,
           *eps = nullptr, *lam = nullptr, *st = nullptr, *hist = nullptr;
    int *perm = nullptr;
    double *h_st = nullptr;   // pinned mirror of st
    cudaGraph_t loop_graph = nullptr;
    cudaGraphExec_t loop_exec = nullptr;
    cudaGraphExec_t step_exec = nullptr;
    unsigned key_mask = 0;
    cudaStream_t key_stream = nullptr;
    int key_shape[3] = {0, 0, 0};
    int mode = 0;             // 1: conditional-graph loop, 2: host-stepped graphs
    int iters = 0;            // iterations of the last run
    bool ready = false;
};

namespace dftg {
namespace {

void scf_drop_graphs(dftg_scf_state *s)
{
    if (s->loop_exec) cudaGraphExecDestroy(s->loop_exec);
    if (s->loop_graph) cudaGraphDestroy(s->loop_graph);
    if (s->step_exec) cudaGraphExecDestroy(s->step_exec);
    s->loop_exec = nullptr;
    s->loop_graph = nullptr;
    s->step_exec = nullptr;
}

GemmOp gop(int m, int n, int k, const double *A, int lda, bool ta, const double *B, int ldb, bool tb, double *C,
           int ldc, double alpha = 1.0, double beta = 0.0, const double *C0 = nullptr, const int *bcol = nullptr)
{
    GemmOp g;
    g.m = m; g.n = n; g.k = k; g.ta = ta; g.tb = tb; g.lda = lda; g.ldb = ldb; g.ldc = ldc;
    g.alpha = alpha; g.beta = beta; g.A = A; g.B = B; g.C0 = C0 ? C0 : C; g.bcol = bcol; g.C = C;
    return g;
}

int gemm(cudaStream_t st, const GemmOp &a, const GemmOp *b = nullptr)
{
    const int mm = std::max(a.m, b ? b->m : 0), nn = std::max(a.n, b ? b->n : 0);
    const dim3 grid((mm + 7) / 8, (nn + 7) / 8, b ? 2 : 1);
    k_scf_gemm<<<grid, 64, 0, st>>>(a, b ? *b : a);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

int jacobi(dftg_ctx *c, dftg_scf_state *s, const double *A, double *V)
{
    k_scf_jacobi<<<1, kJacobiThreads, jacobi_smem(s->n), c->stream>>>(s->n, A, V, s->lam, s->st);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// eigenvectors of A (n x n) refined across the occupied / virtual split;
// returns the buffer holding them (V0 or V1) in *out, eps / perm set.  warm:
// the Jacobi rotations start from the previous solve's vectors Vk (A is
// rotated into that basis first: A_w = Vk^T A Vk, V = Vk V_w), which leaves
// few rotations once the SCF settles; the result is copied back to Vk.
int eigen_solve(dftg_ctx *c, dftg_scf_state *s, const double *A, bool warm, double **out)
{
    const int n = s->n;
    double *cur = s->V0, *nxt = s->V1;
    if (warm) {
        DFTG_TRY_L(gemm(c->stream, gop(n, n, n, A, n, false, s->Vk, n, false, s->T, n)));
        DFTG_TRY_L(gemm(c->stream, gop(n, n, n, s->Vk, n, true, s->T, n, false, s->W, n)));
        DFTG_TRY_L(jacobi(c, s, s->W, nxt));
        DFTG_TRY_L(gemm(c->stream, gop(n, n, n, s->Vk, n, false, nxt, n, false, cur, n)));
    } else {
        DFTG_TRY_L(jacobi(c, s, A, cur));
    }
    for (int r = 0; r < s->nref; ++r) {
        const GemmOp g1 = gop(n, n, n, cur, n, true, cur, n, false, s->G, n);
        const GemmOp g2 = gop(n, n, n, A, n, false, cur, n, false, s->W, n);
        DFTG_TRY_L(gemm(c->stream, g1, &g2));
        DFTG_TRY_L(gemm(c->stream, gop(n, n, n, cur, n, true, s->W, n, false, s->S, n)));
        DFTG_CUDA(cudaMemsetAsync(s->st + kStCross, 0, 2 * sizeof(double), c->stream));
        k_scf_refine<<<(n * n + 255) / 256, 256, 0, c->stream>>>(n, s->nocc, s->G, s->S, s->E, s->eps, s->perm, s->st);
        DFTG_LAUNCH_CHECK();
        DFTG_TRY_L(gemm(c->stream, gop(n, n, n, cur, n, false, s->E, n, false, nxt, n, 1.0, 1.0, cur)));
        std::swap(cur, nxt);
    }
    DFTG_CUDA(cudaMemcpyAsync(s->Vk, cur, sizeof(double) * (size_t)n * n, cudaMemcpyDeviceToDevice, c->stream));
    *out = cur;
    return DFTG_OK;
}

// DFT::calculate_density_matrix (dft.cpp:330-366): P <- w_new C_occ C_occ^T + w_old P
int density_step(dftg_ctx *c, dftg_scf_state *s, double w_new, double w_old, bool warm)
{
    const int n = s->n, n2 = n * n;
    k_scf_axpby<<<(n2 + 255) / 256, 256, 0, c->stream>>>(n2, 1.0, s->H, 2.0, c->d_J, 1.0, c->d_XC, s->F);
    DFTG_LAUNCH_CHECK();
    DFTG_TRY_L(gemm(c->stream, gop(n, n, n, s->F, n, false, s->X, n, false, s->T, n)));
    DFTG_TRY_L(gemm(c->stream, gop(n, n, n, s->X, n, true, s->T, n, false, s->Fp, n)));
    double *Vf = nullptr;
    DFTG_TRY_L(eigen_solve(c, s, s->Fp, warm, &Vf));
    DFTG_TRY_L(gemm(c->stream, gop(n, s->nocc, n, s->X, n, false, Vf, n, false, s->C, n, 1.0, 0.0, nullptr, s->perm)));
    DFTG_TRY_L(gemm(c->stream, gop(n, n, s->nocc, s->C, n, false, s->C, n, true, c->d_P, n, w_new, w_old, c->d_P)));
    return DFTG_OK;
}

int energy(dftg_ctx *c, dftg_scf_state *s, int init, cudaGraphConditionalHandle h, int has_cond)
{
    k_scf_energy<<<1, 256, 0, c->stream>>>(s->n, c->d_P, s->H, c->d_J, c->d_scal, init, c->prec_mask != 0 ? 1 : 0,
                                           s->enuc, s->tol, s->min_iter, s->max_iter, s->st, s->hist, h, has_cond);
    DFTG_LAUNCH_CHECK();
    return DFTG_OK;
}

// one SCF iteration: new P (eigen-solve warm-started from the last one), grid
// Fock build, energy and loop test
int iteration(dftg_ctx *c, dftg_scf_state *s, cudaGraphConditionalHandle h, int has_cond)
{
    DFTG_TRY_L(density_step(c, s, 1.0 - s->alpha, s->alpha, true));
    DFTG_TRY_L(fock_pipeline(c));
    DFTG_TRY_L(energy(c, s, 0, h, has_cond));
    return DFTG_OK;
}

bool key_changed(const dftg_ctx *c, const dftg_scf_state *s)
{
    return s->key_mask != c->prec_mask || s->key_stream != c->stream || s->key_shape[0] != c->tc_grid ||
           s->key_shape[1] != c->ct_grid || s->key_shape[2] != c->ct_nst;
}

// The build kernels allocate and configure themselves on their first eager
// run; a capture needs that done.  J and XC (inputs of the next F) are kept.
int warm_pipeline(dftg_ctx *c, dftg_scf_state *s)
{
    const bool warm = c->pipe_warm && c->pipe_mask == c->prec_mask && c->pipe_stream == c->stream &&
                      c->pipe_shape[0] == c->tc_grid && c->pipe_shape[1] == c->ct_grid &&
                      c->pipe_shape[2] == c->ct_nst;
    if (warm) return DFTG_OK;
    const size_t bytes = sizeof(double) * (size_t)s->n * s->n;
    DFTG_CUDA(cudaMemcpyAsync(s->F, c->d_J, bytes, cudaMemcpyDeviceToDevice, c->stream));
    DFTG_CUDA(cudaMemcpyAsync(s->T, c->d_XC, bytes, cudaMemcpyDeviceToDevice, c->stream));
    DFTG_TRY_L(fock_pipeline_graph(c));
    DFTG_CUDA(cudaMemcpyAsync(c->d_J, s->F, bytes, cudaMemcpyDeviceToDevice, c->stream));
    DFTG_CUDA(cudaMemcpyAsync(c->d_XC, s->T, bytes, cudaMemcpyDeviceToDevice, c->stream));
    return DFTG_OK;
}

int prepare_graphs(dftg_ctx *c, dftg_scf_state *s)
{
    DFTG_TRY_L(warm_pipeline(c, s));
    if (key_changed(c, s)) {
        scf_drop_graphs(s);
        s->key_mask = c->prec_mask;
        s->key_stream = c->stream;
        s->key_shape[0] = c->tc_grid;
        s->key_shape[1] = c->ct_grid;
        s->key_shape[2] = c->ct_nst;
    }
    return DFTG_OK;
}

// the whole loop: a conditional while node whose body is one iteration
int build_loop_graph(dftg_ctx *c, dftg_scf_state *s)
{
    cudaGraph_t g = nullptr;
    DFTG_CUDA(cudaGraphCreate(&g, 0));
    cudaGraphConditionalHandle h;
    cudaError_t e = cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault);
    cudaGraphNodeParams p = {cudaGraphNodeTypeConditional};   // aggregate: the other members zero
    p.conditional.handle = h;
    p.conditional.type = cudaGraphCondTypeWhile;
    p.conditional.size = 1;
    cudaGraphNode_t node;
    if (e == cudaSuccess) e = cudaGraphAddNode(&node, g, nullptr, nullptr, 0, &p);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "conditional graph node", __FILE__, __LINE__);
    }
    cudaGraph_t body = p.conditional.phGraph_out[0];
    e = cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaStreamBeginCaptureToGraph", __FILE__, __LINE__);
    }
    const int rc = iteration(c, s, h, 1);
    cudaGraph_t captured = nullptr;
    e = cudaStreamEndCapture(c->stream, &captured);
    if (rc != DFTG_OK || e != cudaSuccess) {
        cudaGraphDestroy(g);
        return rc != DFTG_OK ? rc : cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    }
    e = cudaGraphInstantiate(&s->loop_exec, g, 0);
    if (e != cudaSuccess) {
        s->loop_exec = nullptr;
        cudaGraphDestroy(g);
        return cuda_fail(e, "cudaGraphInstantiate (conditional loop)", __FILE__, __LINE__);
    }
    s->loop_graph = g;
    return DFTG_OK;
}

int build_step_graph(dftg_ctx *c, dftg_scf_state *s)
{
    cudaGraph_t g = nullptr;
    DFTG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    const int rc = iteration(c, s, 0, 0);
    const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc != DFTG_OK || e != cudaSuccess) {
        if (g) cudaGraphDestroy(g);
        return rc != DFTG_OK ? rc : cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
    }
    const cudaError_t ei = cudaGraphInstantiate(&s->step_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) {
        s->step_exec = nullptr;
        return cuda_fail(ei, "cudaGraphInstantiate (SCF step)", __FILE__, __LINE__);
    }
    return DFTG_OK;
}

int read_state(dftg_ctx *c, dftg_scf_state *s)
{
    DFTG_CUDA(cudaMemcpyAsync(s->h_st, s->st, sizeof(double) * kStElems, cudaMemcpyDeviceToHost, c->stream));
    DFTG_TRY_L(sync_scalars(c));   // synchronises; reports an expired bounded wait
    return DFTG_OK;
}

void mark_built(dftg_ctx *c)
{
    c->have_density = true;
    c->have_hartree = true;
    c->have_build = true;
    c->fwd_mask = c->prec_mask;
    c->rho_scaled = true;
}

}  // namespace

void scf_free(dftg_ctx *c)
{
    dftg_scf_state *s = c->scf;
    if (!s) return;
    scf_drop_graphs(s);
    if (s->buf) cudaFree(s->buf);
    if (s->perm) cudaFree(s->perm);
    if (s->h_st) cudaFreeHost(s->h_st);
    delete s;
    c->scf = nullptr;
}

}  // namespace dftg

using namespace dftg;

extern "C" int dftg_scf_init(dftg_ctx *c, const dftg_scf_params *prm)
{
    if (!c || !prm) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    if (c->points_only) { set_error("a point-set context has no nuclei: no SCF"); return DFTG_ERR_STATE; }
    if (c->cell0 != 0 || c->ncell != c->natoms) { set_error("a context over part of the cells has no whole build: no SCF"); return DFTG_ERR_STATE; }
    const int n = c->nbf;
    if (n > kScfMaxN) {
        set_error("device SCF supports nbf <= %d (got %d)", kScfMaxN, n);
        return DFTG_ERR_ARG;
    }
    int nelec = prm->nelec;
    if (nelec == 0)
        for (int z : c->Z) nelec += z;
    if (nelec <= 0 || (nelec & 1) || nelec / 2 > n) {
        set_error("nelec %d: closed shell needs an even count with nelec / 2 <= nbf", nelec);
        return DFTG_ERR_ARG;
    }
    if (!(prm->alpha >= 0.0 && prm->alpha < 1.0) || !(prm->tol >= 0.0) || prm->min_iter < 0 || prm->max_iter < 1 ||
        prm->max_iter > DFTG_SCF_MAX_ITER || prm->refine_steps < 0 || prm->refine_steps > 16) {
        set_error("invalid SCF parameters (alpha in [0,1), tol >= 0, 1 <= max_iter <= %d, refine_steps <= 16)",
                  DFTG_SCF_MAX_ITER);
        return DFTG_ERR_ARG;
    }
    DFTG_CUDA(cudaSetDevice(c->device));
    scf_free(c);
    dftg_scf_state *s = new dftg_scf_state();
    c->scf = s;
    s->n = n;
    s->nocc = nelec / 2;
    s->nref = prm->refine_steps ? prm->refine_steps : kRefineDefault;
    s->alpha = prm->alpha;
    s->tol = prm->tol;
    s->min_iter = prm->min_iter;
    s->max_iter = prm->max_iter;
    const size_t n2 = (size_t)n * n;
    const size_t total = 14 * n2 + 2 * (size_t)n + kStElems + (size_t)kHistW * s->max_iter;
    int rc = DFTG_OK;
#define SCF_CUDA(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) { rc = cuda_fail(e_, #call, __FILE__, __LINE__); scf_free(c); return rc; } } while (0)
#define SCF_TRY(x) do { rc = (x); if (rc != DFTG_OK) { scf_free(c); return rc; } } while (0)
    SCF_CUDA(cudaMalloc(&s->buf, sizeof(double) * total));
    SCF_CUDA(cudaMalloc(&s->perm, sizeof(int) * n));
    SCF_CUDA(cudaMallocHost(&s->h_st, sizeof(double) * kStElems));
    double *p = s->buf;
    double **mats[] = {&s->H, &s->X, &s->X2, &s->F, &s->T, &s->Fp, &s->V0, &s->V1, &s->Vk, &s->G, &s->W, &s->S, &s->E};
    for (double **m : mats) { *m = p; p += n2; }
    s->C = p; p += n2;
    s->eps = p; p += n;
    s->lam = p; p += n;
    s->st = p; p += kStElems;
    s->hist = p;
    SCF_CUDA(cudaMemsetAsync(s->buf, 0, sizeof(double) * total, c->stream));
    rc = allow_max_dyn_smem((const void *)k_scf_jacobi, c->device);
    if (rc != DFTG_OK) { scf_free(c); return rc; }
    SCF_TRY(dftg_nuclear_repulsion(c, &s->enuc));

    // S, T, V and H = T + V (dft.cpp:184-199)
    if (!c->d_ints_work) SCF_CUDA(cudaMalloc(&c->d_ints_work, 3 * n2 * sizeof(double)));
    double *dS = c->d_ints_work, *dT = dS + n2, *dV = dT + n2;
    SCF_TRY(launch_one_electron(c, dS, dT, dV));
    k_scf_axpby<<<((int)n2 + 255) / 256, 256, 0, c->stream>>>((int)n2, 1.0, dT, 1.0, dV, 0.0, nullptr, s->H);
    SCF_CUDA(cudaGetLastError());

    // X with X^T S X = I (dft.cpp:300-316)
    SCF_TRY(jacobi(c, s, dS, s->V0));
    SCF_CUDA(cudaMemcpyAsync(s->h_st, s->st, sizeof(double) * kStElems, cudaMemcpyDeviceToHost, c->stream));
    SCF_CUDA(cudaStreamSynchronize(c->stream));
    if (!(s->h_st[kStLamMin] > 0.0)) {
        set_error("overlap matrix not positive definite (smallest eigenvalue %g)", s->h_st[kStLamMin]);
        scf_free(c);
        return DFTG_ERR_STATE;
    }
    k_scf_scale_cols<<<((int)n2 + 255) / 256, 256, 0, c->stream>>>(n, s->V0, s->lam, s->X);
    SCF_CUDA(cudaGetLastError());
    for (int it = 0; it < kNsSteps; ++it) {
        SCF_TRY(gemm(c->stream, gop(n, n, n, dS, n, false, s->X, n, false, s->T, n)));
        SCF_TRY(gemm(c->stream, gop(n, n, n, s->X, n, true, s->T, n, false, s->G, n)));
        SCF_TRY(gemm(c->stream, gop(n, n, n, s->X, n, false, s->G, n, false, s->X2, n, -0.5, 1.5, s->X)));
        std::swap(s->X, s->X2);
    }

    // first density from H, its J, E_0 with E_xc = 0 (dft.cpp:216-226)
    SCF_CUDA(cudaMemsetAsync(c->d_J, 0, sizeof(double) * n2, c->stream));
    SCF_CUDA(cudaMemsetAsync(c->d_XC, 0, sizeof(double) * n2, c->stream));
    SCF_TRY(density_step(c, s, 1.0, 0.0, false));
    SCF_TRY(fock_pipeline_graph(c));
    SCF_CUDA(cudaMemsetAsync(c->d_XC, 0, sizeof(double) * n2, c->stream));
    SCF_TRY(energy(c, s, 1, 0, 0));
    SCF_TRY(read_state(c, s));
    mark_built(c);
    s->iters = 0;
    s->ready = true;
#undef SCF_CUDA
#undef SCF_TRY
    return DFTG_OK;
}

extern "C" int dftg_scf_run(dftg_ctx *c, double *energy_out, int *iterations)
{
    if (!c || !c->scf || !c->scf->ready) { set_error("dftg_scf_init first"); return DFTG_ERR_STATE; }
    dftg_scf_state *s = c->scf;
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY_L(prepare_graphs(c, s));
    if (!s->loop_exec && s->mode != 2) {
        if (build_loop_graph(c, s) == DFTG_OK) {
            s->mode = 1;
        } else {
            cudaGetLastError();
            s->mode = 2;   // no conditional nodes here: one graph launch per iteration
        }
    }
    DFTG_CUDA(cudaMemsetAsync(s->st + kStIt, 0, sizeof(double), c->stream));
    if (s->mode == 1) {
        DFTG_CUDA(cudaGraphLaunch(s->loop_exec, c->stream));
        DFTG_TRY_L(read_state(c, s));
    } else {
        if (!s->step_exec) DFTG_TRY_L(build_step_graph(c, s));
        for (int it = 0; it < s->max_iter; ++it) {
            DFTG_CUDA(cudaGraphLaunch(s->step_exec, c->stream));
            DFTG_TRY_L(read_state(c, s));
            if (s->h_st[kStCont] == 0.0) break;
        }
    }
    mark_built(c);
    s->iters = (int)s->h_st[kStIt];
    if (energy_out) *energy_out = s->h_st[kStE];
    if (iterations) *iterations = s->iters;
    return DFTG_OK;
}

extern "C" int dftg_scf_step(dftg_ctx *c, double *energy_out, int *converged)
{
    if (!c || !c->scf || !c->scf->ready) { set_error("dftg_scf_init first"); return DFTG_ERR_STATE; }
    dftg_scf_state *s = c->scf;
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY_L(prepare_graphs(c, s));
    if (!s->step_exec) DFTG_TRY_L(build_step_graph(c, s));
    DFTG_CUDA(cudaGraphLaunch(s->step_exec, c->stream));
    DFTG_TRY_L(read_state(c, s));
    mark_built(c);
    s->iters = std::min((int)s->h_st[kStIt], s->max_iter);
    if (energy_out) *energy_out = s->h_st[kStE];
    if (converged) *converged = s->h_st[kStCont] == 0.0 ? 1 : 0;
    return DFTG_OK;
}

extern "C" int dftg_scf_get(dftg_ctx *c, int what, double *out, size_t cap, size_t *nout)
{
    if (!c || !c->scf || !c->scf->ready) { set_error("dftg_scf_init first"); return DFTG_ERR_STATE; }
    if (!out) { set_error("out NULL"); return DFTG_ERR_ARG; }
    dftg_scf_state *s = c->scf;
    const size_t n2 = (size_t)s->n * s->n;
    const double *src = nullptr;
    size_t cnt = 0;
    switch (what) {
    case DFTG_SCF_P: src = c->d_P; cnt = n2; break;
    case DFTG_SCF_J: src = c->d_J; cnt = n2; break;
    case DFTG_SCF_XC: src = c->d_XC; cnt = n2; break;
    case DFTG_SCF_H: src = s->H; cnt = n2; break;
    case DFTG_SCF_X: src = s->X; cnt = n2; break;
    case DFTG_SCF_EPS: src = s->eps; cnt = s->n; break;
    case DFTG_SCF_COCC: src = s->C; cnt = (size_t)s->n * s->nocc; break;
    case DFTG_SCF_HISTORY: src = s->hist; cnt = (size_t)kHistW * s->iters; break;
    case DFTG_SCF_DIAG:
    case DFTG_SCF_STATE: {
        if (cap < 4) { set_error("cap %zu < 4", cap); return DFTG_ERR_ARG; }
        DFTG_CUDA(cudaSetDevice(c->device));
        DFTG_CUDA(cudaMemcpyAsync(s->h_st, s->st, sizeof(double) * kStElems, cudaMemcpyDeviceToHost, c->stream));
        DFTG_CUDA(cudaStreamSynchronize(c->stream));
        const double *h = s->h_st;
        if (what == DFTG_SCF_DIAG) {
            out[0] = h[kStCross]; out[1] = h[kStOrth]; out[2] = h[kStSweeps]; out[3] = s->mode;
        } else {
            out[0] = h[kStE]; out[1] = h[kStIt]; out[2] = h[kStDiff]; out[3] = h[kStCont];
        }
        if (nout) *nout = 4;
        return DFTG_OK;
    }
    default: set_error("unknown SCF output %d", what); return DFTG_ERR_ARG;
    }
    if (cap < cnt) { set_error("cap %zu < %zu", cap, cnt); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    if (cnt) DFTG_CUDA(cudaMemcpyAsync(out, src, sizeof(double) * cnt, cudaMemcpyDeviceToHost, c->stream));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    if (nout) *nout = cnt;
    return DFTG_OK;
}
