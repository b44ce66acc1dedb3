// dftg_capi.cu -- extern "C" entry points of include/dftg.h.
//
// Owns the context (device buffers, stream, call-order state) and sequences the
// kernels of one grid Fock build:
//   set_density      K3 rho = 2 phi^T P phi              (gridpoint.cpp:82-84)
//   correct_density  K6 c = sum Z / int w rho, rho *= c   (moleculargrid.cpp:132-146)
//   xc points        LDA point kernel, cxc = w v_xc, E_xc (dft.cpp:394-424)
//   hartree          K5a-e, cj = w V / 2                  (moleculargrid.cpp:336-380)
//   contraction      K4 XC and J in one pass over phi     (dft.cpp:426-432, atomicgrid.cpp:471-488)
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <mutex>
#include <vector>
#include "dftg_internal.cuh"
#include "lebedev_data.h"

namespace dftg {

static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what, const char *file, int line)
{
    set_error("CUDA error %s (%s) at %s:%d in %s", cudaGetErrorName(e), cudaGetErrorString(e), file, line, what);
    return e == cudaErrorMemoryAllocation ? DFTG_ERR_NOMEM : DFTG_ERR_CUDA;
}

int mark(dftg_ctx *c, const char *name)
{
    if (c->prof_n >= dftg_ctx::kMaxMarks) return DFTG_OK;
    cudaEvent_t &ev = c->prof_ev[c->prof_n];
    if (!ev) DFTG_CUDA(cudaEventCreate(&ev));
    DFTG_CUDA(cudaEventRecord(ev, c->stream));
    c->prof_name[c->prof_n] = name;
    ++c->prof_n;
    return DFTG_OK;
}

static double dfact(int n) { double r = 1.0; for (int k = n; k > 1; k -= 2) r *= k; return r; }

// GTO normalisation constant, cgf.cpp:102-114 (truncated pi of cgf.cpp:103)
double gto_norm(double alpha, int l, int m, int n)
{
    double nom = std::pow(2.0, 2.0 * (l + m + n) + 3.0 / 2.0) * std::pow(alpha, (l + m + n) + 3.0 / 2.0);
    double denom = (l < 1 ? 1 : dfact(2 * l - 1)) * (m < 1 ? 1 : dfact(2 * m - 1)) * (n < 1 ? 1 : dfact(2 * n - 1)) *
                   std::pow(kPiTrunc, 3.0 / 2.0);
    return std::sqrt(nom / denom);
}

template <typename T>
static int dalloc(T **p, size_t n)
{
    if (n == 0) n = 1;
    DFTG_CUDA(cudaMalloc(reinterpret_cast<void **>(p), n * sizeof(T)));
    return DFTG_OK;
}

#define DFTG_TRY(x) do { int rc_ = (x); if (rc_ != DFTG_OK) return rc_; } while (0)

static void free_ctx(dftg_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    void *bufs[] = {c->d_atoms, c->d_rab, c->d_rn, c->d_wrad, c->d_leb, c->d_bf_lmn, c->d_bf_off, c->d_bf_atom,
                    c->d_pa, c->d_pcn, c->d_x, c->d_y, c->d_z, c->d_w, c->d_wb, c->d_rho, c->d_V, c->d_Vown,
                    c->d_cxc, c->d_cj, c->d_cxc32, c->d_cj32, c->d_phi, c->d_phi32, c->d_P, c->d_P32, c->d_J,
                    c->d_XC, c->d_part, c->d_red, c->d_scal, c->d_Y, c->d_Yw, c->d_pre, c->d_pre32, c->d_rec,
                    c->d_rec32, c->d_rholm, c->d_U, c->d_U32, c->d_Y32, c->d_Ywt32, c->d_fold, c->d_Gt,
                    c->d_Gb, c->d_Kt, c->d_sx, c->d_splf, c->d_spl, c->d_splm, c->d_tiles,
                    c->d_ints_work, c->d_tcA, c->d_tcB, c->d_tc_rowexp, c->d_tc_colexp, c->d_sgrid, c->d_rw32, c->d_wsplit, c->d_lebpair, c->d_flag,
                    c->d_pairs, c->d_pairpos, c->d_pairv, c->d_cross_tasks, c->d_ct_rowexp, c->d_ct_A, c->d_ct_winv, c->d_ct_cmax, c->d_counters, c->d_invr, c->d_maps32, c->d_U32T,
                    c->d_bw_pt, c->d_bw_lm, c->d_bw_fpart, c->d_bw_out, c->d_bw_counter, c->d_bw_pairp,
                    c->d_bw_binfirst, c->d_bw_cpart, c->d_bw_geo, c->d_bw_geo64, c->d_bw_prim32,
                    c->d_tt_exp, c->d_tt_winv, c->d_tt_A, c->d_tt_B, c->d_tt_part,
                    c->d_dt_A, c->d_dt_B, c->d_dt_exp};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (c->h_scal) cudaFreeHost(c->h_scal);
    if (c->pipe_exec) cudaGraphExecDestroy(c->pipe_exec);
    scf_free(c);
    for (cudaEvent_t ev : c->prof_ev)
        if (ev) cudaEventDestroy(ev);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    if (c->aux_stream) cudaStreamDestroy(c->aux_stream);
    if (c->ev_fork) cudaEventDestroy(c->ev_fork);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    delete c;
}

// DFTG_TRACE=1: wall time of each set-up phase on stderr (the stream is
// synchronised at every mark, so GPU work is charged to its phase)
struct SetupTrace {
    bool on = false;
    std::chrono::steady_clock::time_point t0;
    SetupTrace()
    {
        const char *e = std::getenv("DFTG_TRACE");
        on = e && e[0] == '1';
        t0 = std::chrono::steady_clock::now();
    }
    void mark(cudaStream_t st, const char *what)
    {
        if (!on) return;
        if (st) cudaStreamSynchronize(st);
        const auto t = std::chrono::steady_clock::now();
        std::fprintf(stderr, "dftg set-up %-22s %9.3f ms\n", what, std::chrono::duration<double, std::milli>(t - t0).count());
        t0 = t;
    }
};

static int build_ctx(dftg_ctx *c, const dftg_molecule *mol, const dftg_basis *basis, const dftg_grid_params *g,
                     int cell0 = 0, int ncell = -1)
{
    SetupTrace tr;
    c->device = g->device;
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
    tr.mark(c->stream, "stream");

    // molecule and basis
    c->natoms = mol->natoms;
    c->Z.assign(mol->Z, mol->Z + mol->natoms);
    c->xyz.assign(mol->xyz, mol->xyz + 3 * mol->natoms);
    c->nbf = basis->nbf;
    c->bf_atom.assign(basis->bf_atom, basis->bf_atom + c->nbf);
    c->bf_lmn.assign(basis->bf_lmn, basis->bf_lmn + 3 * c->nbf);
    c->bf_off.assign(c->nbf + 1, 0);
    for (int i = 0; i < c->nbf; ++i) c->bf_off[i + 1] = c->bf_off[i] + basis->bf_nprim[i];
    c->nprim = c->bf_off[c->nbf];
    c->alpha.assign(basis->prim_alpha, basis->prim_alpha + c->nprim);
    c->coef.assign(basis->prim_coef, basis->prim_coef + c->nprim);
    c->norm.resize(c->nprim);
    std::vector<double> pcn(c->nprim);
    for (int i = 0; i < c->nbf; ++i)
        for (int k = c->bf_off[i]; k < c->bf_off[i + 1]; ++k) {
            c->norm[k] = gto_norm(c->alpha[k], c->bf_lmn[3 * i], c->bf_lmn[3 * i + 1], c->bf_lmn[3 * i + 2]);
            pcn[k] = c->coef[k] * c->norm[k];
        }

    // radial grid, atomicgrid.cpp:44-63
    c->nrad = g->radial_points;
    c->leb = g->lebedev_order;
    c->nang = dftg_lebedev_npts[c->leb];
    c->lmax = g->lmax;
    c->nlm = (c->lmax + 1) * (c->lmax + 1);
    c->cell0 = cell0;
    c->ncell = ncell < 0 ? c->natoms : ncell;
    c->npts = (size_t)c->ncell * c->nrad * c->nang;
    c->npad = (c->npts + kPtsAlign - 1) / kPtsAlign * kPtsAlign;
    c->r_n.resize(c->nrad);
    c->w_rad.resize(c->nrad);
    const double f = kPi / (double)(c->nrad + 1);
    for (int p = 1; p <= c->nrad; ++p) {
        double w = f * std::pow(std::sin(f * (double)p), 2.0);
        const double x = std::cos(f * (double)p);
        c->r_n[p - 1] = (1.0 + x) / (1.0 - x);
        w = w / std::sqrt(1.0 - std::pow(x, 2.0)) * 2.0 / std::pow(1.0 - x, 2.0);
        c->w_rad[p - 1] = w;
    }

    const size_t np = c->npad, nn = (size_t)c->nbf * c->nbf, nlm = c->nlm, N = c->nrad;
    tr.mark(nullptr, "host basis and radial grid");
    DFTG_TRY(dalloc(&c->d_atoms, 4 * (size_t)c->natoms));
    DFTG_TRY(dalloc(&c->d_rab, (size_t)c->natoms * c->natoms));
    DFTG_TRY(dalloc(&c->d_rn, N));
    DFTG_TRY(dalloc(&c->d_wrad, N));
    DFTG_TRY(dalloc(&c->d_leb, 4 * (size_t)c->nang));
    DFTG_TRY(dalloc(&c->d_bf_lmn, 3 * (size_t)c->nbf));
    DFTG_TRY(dalloc(&c->d_bf_off, (size_t)c->nbf + 1));
    DFTG_TRY(dalloc(&c->d_bf_atom, (size_t)c->nbf));
    DFTG_TRY(dalloc(&c->d_pa, (size_t)c->nprim));
    DFTG_TRY(dalloc(&c->d_pcn, (size_t)c->nprim));
    DFTG_TRY(dalloc(&c->d_x, np));
    DFTG_TRY(dalloc(&c->d_y, np));
    DFTG_TRY(dalloc(&c->d_z, np));
    DFTG_TRY(dalloc(&c->d_w, np));
    DFTG_TRY(dalloc(&c->d_wb, np));
    DFTG_TRY(dalloc(&c->d_rho, np));
    DFTG_CUDA(cudaMalloc(&c->d_rw32, sizeof(float) * 2 * np));
    DFTG_CUDA(cudaMalloc(&c->d_wsplit, sizeof(float) * 4 * np));
    DFTG_TRY(dalloc(&c->d_V, np));
    DFTG_TRY(dalloc(&c->d_Vown, np));
    DFTG_TRY(dalloc(&c->d_cxc, np));
    DFTG_TRY(dalloc(&c->d_cj, np));
    DFTG_TRY(dalloc(&c->d_cxc32, np));
    DFTG_TRY(dalloc(&c->d_cj32, np));
    DFTG_TRY(dalloc(&c->d_phi, np * c->nbf));
    DFTG_TRY(dalloc(&c->d_phi32, np * c->nbf));
    DFTG_TRY(dalloc(&c->d_P, nn));
    DFTG_TRY(dalloc(&c->d_P32, 2 * (size_t)c->nbf * ((c->nbf + 3) / 4 * 4)));   // FP32 hi, lo of P, rows padded to 4
    DFTG_TRY(dalloc(&c->d_J, nn));
    DFTG_TRY(dalloc(&c->d_XC, nn));
    int nsm = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    size_t part = contract_part_elems(c->nbf, c->npad);
    const size_t part_tc = contract_tc_part_elems(c->nbf, c->npad, nsm);
    if (part_tc > part) part = part_tc;
    const size_t spline_work = 2 * (size_t)c->natoms * nlm * N;
    c->part_elems = part > spline_work ? part : spline_work;
    DFTG_TRY(dalloc(&c->d_part, c->part_elems));
    c->red_lda_off = reduction_elems(c->npad, c->natoms, c->nrad, c->nang) + 64;
    c->red_elems = c->red_lda_off + 2 * lda_blocks(c->npad);
    DFTG_TRY(dalloc(&c->d_red, c->red_elems));
    DFTG_TRY(dalloc(&c->d_scal, scal_elems(c->natoms)));
    DFTG_CUDA(cudaMalloc(&c->d_counters, sizeof(int) * kNumCounters));
    DFTG_CUDA(cudaMemset(c->d_counters, 0, sizeof(int) * kNumCounters));
    DFTG_CUDA(cudaMallocHost(&c->h_scal, sizeof(double) * (scal_elems(c->natoms) + 1)));   // + the wait flag
    DFTG_TRY(dalloc(&c->d_Y, nlm * c->nang));
    DFTG_TRY(dalloc(&c->d_Yw, nlm * c->nang));
    DFTG_TRY(dalloc(&c->d_pre, nlm));
    DFTG_TRY(dalloc(&c->d_pre32, nlm));
    DFTG_TRY(dalloc(&c->d_rec, 2 * nlm));
    DFTG_TRY(dalloc(&c->d_rec32, 2 * nlm));
    DFTG_TRY(dalloc(&c->d_rholm, (size_t)c->natoms * nlm * N));
    DFTG_TRY(dalloc(&c->d_U, (size_t)c->natoms * nlm * N));
    DFTG_TRY(dalloc(&c->d_U32, 2 * (size_t)c->natoms * nlm * N));
    DFTG_TRY(dalloc(&c->d_U32T, 2 * (size_t)c->natoms * nlm * N));
    DFTG_TRY(dalloc(&c->d_Y32, 2 * nlm * c->nang));
    DFTG_TRY(dalloc(&c->d_Ywt32, 2 * nlm * c->nang));
    DFTG_TRY(dalloc(&c->d_fold, nlm));
    DFTG_TRY(dalloc(&c->d_sx, N));
    DFTG_TRY(dalloc(&c->d_splf, hartree_splf_elems(c->nrad)));
    DFTG_TRY(dalloc(&c->d_spl, (size_t)c->natoms * nlm * N * 4));
    DFTG_TRY(dalloc(&c->d_splm, (size_t)c->natoms * nlm * N * 8));
    DFTG_CUDA(cudaMemset(c->d_scal, 0, sizeof(double) * scal_elems(c->natoms)));

    tr.mark(c->stream, "allocations");
    std::vector<double> atoms(4 * (size_t)c->natoms), rab((size_t)c->natoms * c->natoms);
    for (int a = 0; a < c->natoms; ++a) {
        for (int d = 0; d < 3; ++d) atoms[4 * a + d] = c->xyz[3 * a + d];
        atoms[4 * a + 3] = (double)c->Z[a];
    }
    for (int a = 0; a < c->natoms; ++a)
        for (int b = 0; b < c->natoms; ++b) {
            double dx = c->xyz[3 * b] - c->xyz[3 * a], dy = c->xyz[3 * b + 1] - c->xyz[3 * a + 1],
                   dz = c->xyz[3 * b + 2] - c->xyz[3 * a + 2];
            rab[(size_t)a * c->natoms + b] = std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    DFTG_CUDA(cudaMemcpy(c->d_atoms, atoms.data(), sizeof(double) * atoms.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_rab, rab.data(), sizeof(double) * rab.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_rn, c->r_n.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_wrad, c->w_rad.data(), sizeof(double) * N, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_leb, dftg_lebedev_table[dftg_lebedev_offset[c->leb]], sizeof(double) * 4 * c->nang,
                         cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_bf_lmn, c->bf_lmn.data(), sizeof(int) * 3 * c->nbf, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_bf_off, c->bf_off.data(), sizeof(int) * (c->nbf + 1), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_bf_atom, c->bf_atom.data(), sizeof(int) * c->nbf, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_pa, c->alpha.data(), sizeof(double) * c->nprim, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_pcn, pcn.data(), sizeof(double) * c->nprim, cudaMemcpyHostToDevice));

    tr.mark(c->stream, "copies");
    DFTG_TRY(launch_grid(c));
    DFTG_TRY(launch_weight_planes(c));
    tr.mark(c->stream, "grid and Becke weights");
    DFTG_TRY(launch_amplitudes(c));
    tr.mark(c->stream, "amplitudes");
    DFTG_TRY(hartree_setup(c));
    tr.mark(c->stream, "Hartree maps");
    DFTG_TRY(contract_setup(c));
    tr.mark(c->stream, "contraction tiles");
    DFTG_TRY(contract_tc_setup(c));
    DFTG_TRY(contract_tt_setup(c));
    tr.mark(c->stream, "contraction slices");
    DFTG_TRY(density_tc_setup(c));
    DFTG_TRY(density_tt_setup(c));
    tr.mark(c->stream, "density slices");
    DFTG_TRY(cross_pairs_setup(c));
    tr.mark(c->stream, "cross-atom pairs");
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    return DFTG_OK;
}

int allow_max_dyn_smem(const void *func, int device)
{
    static std::mutex mu;
    static std::vector<std::pair<const void *, int>> done;
    std::lock_guard<std::mutex> lock(mu);
    for (const auto &d : done)
        if (d.first == func && d.second == device) return DFTG_OK;
    int optin = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, device));
    cudaFuncAttributes fa{};
    DFTG_CUDA(cudaFuncGetAttributes(&fa, func));
    DFTG_CUDA(cudaFuncSetAttribute(func, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes));
    done.emplace_back(func, device);
    return DFTG_OK;
}

static int check_matrix(const double *P, int n)
{
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const double a = P[i + (size_t)j * n];
            if (!std::isfinite(a)) {
                set_error("P(%d,%d) is not finite", i, j);
                return DFTG_ERR_NONFINITE;
            }
            const double b = P[j + (size_t)i * n];
            if (std::fabs(a - b) > 1e-10 * (1.0 + std::fabs(a))) {
                set_error("P is not symmetric at (%d,%d): %g vs %g", i, j, a, b);
                return DFTG_ERR_NONFINITE;
            }
        }
    return DFTG_OK;
}

int sync_scalars(dftg_ctx *c)
{
    const size_t ns = scal_elems(c->natoms);
    int *h_flag = reinterpret_cast<int *>(c->h_scal + ns);   // pinned slot after the scalars
    DFTG_CUDA(cudaMemcpyAsync(c->h_scal, c->d_scal, sizeof(double) * ns, cudaMemcpyDeviceToHost, c->stream));
    if (c->d_flag) DFTG_CUDA(cudaMemcpyAsync(h_flag, c->d_flag, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    if (c->d_flag && *h_flag) {   // a bounded wait inside a kernel gave up
        const int flag = *h_flag;
        DFTG_CUDA(cudaMemset(c->d_flag, 0, sizeof(int)));
        *h_flag = 0;
        set_error("a bounded device wait expired (code %d); results of this build are invalid", flag);
        return DFTG_ERR_TIMEOUT;
    }
    return DFTG_OK;
}

// device part of one Fock build; P already in c->d_P
int fock_pipeline(dftg_ctx *c)
{
    // the steps made inside take the whole build's forms (cmax_route)
    struct WholeBuild {
        dftg_ctx *c;
        ~WholeBuild() { c->whole_build = false; }
    } whole{c};
    c->whole_build = true;
    const bool fused = sgrid_route(c);
    DFTG_TRY(launch_density(c, fused));
    if (!fused) {
        DFTG_TRY(launch_atom_sums(c, kSumsFactor));
        // rescales rho by the correction factor; with the mixed point kernel it also
        // sums the corrected N and writes the rho w_becke planes of the multipoles
        DFTG_TRY(launch_xc_points(c, true, (c->prec_mask & kPrecLda) != 0));
        c->rho_scaled = true;
        DFTG_TRY(launch_hartree(c));
    } else {
        // the correction factor came from the P-slicing step (2 tr(P S_grid)) and
        // the density epilogue applied it and wrote the rho w_becke planes, so the
        // LDA point kernel and the Hartree steps are independent: the Hartree
        // steps (the longer branch) run on a second stream of the greatest
        // priority beside the point kernel (not when the phases are being timed)
        c->rho_scaled = true;
        const bool fork = !c->prof_on;
        const cudaStream_t main = c->stream;
        if (fork) {
            if (!c->aux_stream) {
                int least = 0, greatest = 0;
                DFTG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
                DFTG_CUDA(cudaStreamCreateWithPriority(&c->aux_stream, cudaStreamNonBlocking, greatest));
            }
            if (!c->ev_fork) DFTG_CUDA(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
            if (!c->ev_join) DFTG_CUDA(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
            DFTG_CUDA(cudaEventRecord(c->ev_fork, main));
            DFTG_CUDA(cudaStreamWaitEvent(c->aux_stream, c->ev_fork, 0));
        }
        DFTG_TRY(launch_xc_points(c, false, true, false));
        c->rw_ready = rw_planes(c);
        if (fork) c->stream = c->aux_stream;
        const int rc = launch_hartree(c);
        c->stream = main;
        DFTG_TRY(rc);
        if (fork) {
            DFTG_CUDA(cudaEventRecord(c->ev_join, c->aux_stream));
            DFTG_CUDA(cudaStreamWaitEvent(main, c->ev_join, 0));
        }
    }
    DFTG_TRY(launch_contract(c, true, true));
    return DFTG_OK;
}

// One build on the device buffers (d_P in; d_J, d_XC, d_scal out).  The kernel
// sequence of a (precision mask, stream) pair is captured once into a CUDA
// graph and replayed; the first build of each pair runs eagerly.
static bool pipe_shape_changed(const dftg_ctx *c)
{
    return c->pipe_shape[0] != c->tc_grid || c->pipe_shape[1] != c->ct_grid || c->pipe_shape[2] != c->ct_nst;
}

int fock_pipeline_graph(dftg_ctx *c)
{
    if (c->pipe_exec && (c->pipe_mask != c->prec_mask || c->pipe_stream != c->stream || pipe_shape_changed(c))) {
        cudaGraphExecDestroy(c->pipe_exec);
        c->pipe_exec = nullptr;
        c->pipe_warm = false;
    }
    if (!c->pipe_exec) {
        if (!c->pipe_warm || c->pipe_mask != c->prec_mask || c->pipe_stream != c->stream || pipe_shape_changed(c)) {
            c->pipe_warm = true;
            c->pipe_mask = c->prec_mask;
            c->pipe_stream = c->stream;
            c->pipe_shape[0] = c->tc_grid;
            c->pipe_shape[1] = c->ct_grid;
            c->pipe_shape[2] = c->ct_nst;
            return fock_pipeline(c);
        }
        cudaGraph_t g = nullptr;
        DFTG_CUDA(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
        const int rc = fock_pipeline(c);
        const cudaError_t e = cudaStreamEndCapture(c->stream, &g);
        if (rc != DFTG_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        // node priorities: the Hartree branch's stream priority is kept
        const cudaError_t ei = cudaGraphInstantiate(&c->pipe_exec, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            c->pipe_exec = nullptr;
            return cuda_fail(ei, "cudaGraphInstantiate", __FILE__, __LINE__);
        }
    }
    DFTG_CUDA(cudaGraphLaunch(c->pipe_exec, c->stream));
    c->rho_scaled = true;
    return DFTG_OK;
}

}  // namespace dftg

using namespace dftg;

#define CHECK_CTX(c)                                                   \
    do {                                                               \
        if (!(c)) { set_error("null context"); return DFTG_ERR_ARG; }  \
    } while (0)

// a context over part of the molecule's cells builds only through dftg_shard_*
#define CHECK_WHOLE(c)                                                                                         \
    do {                                                                                                       \
        if ((c)->cell0 != 0 || (c)->ncell != (c)->natoms) {                                                    \
            set_error("the context holds cells [%d, %d) of %d atoms: build it with the dftg_shard_* calls",     \
                      (c)->cell0, (c)->cell0 + (c)->ncell, (c)->natoms);                                        \
            return DFTG_ERR_STATE;                                                                             \
        }                                                                                                      \
    } while (0)

extern "C" {

const char *dftg_last_error(void) { return g_err; }

static int create_checked(const dftg_molecule *mol, const dftg_basis *basis, const dftg_grid_params *g, int cell0,
                          int ncell, dftg_ctx **out);

int dftg_create(const dftg_molecule *mol, const dftg_basis *basis, const dftg_grid_params *g, dftg_ctx **out)
{
    return create_checked(mol, basis, g, 0, -1, out);
}

int dftg_create_cells(const dftg_molecule *mol, const dftg_basis *basis, const dftg_grid_params *g, int first_cell,
                      int ncells, dftg_ctx **out)
{
    if (out) *out = nullptr;
    if (!mol) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    if (first_cell < 0 || ncells < 1 || first_cell + ncells > mol->natoms) {
        set_error("cells [%d, %d) outside the molecule's %d atoms", first_cell, first_cell + ncells, mol->natoms);
        return DFTG_ERR_ARG;
    }
    return create_checked(mol, basis, g, first_cell, ncells, out);
}

static int create_checked(const dftg_molecule *mol, const dftg_basis *basis, const dftg_grid_params *g, int cell0,
                          int ncell, dftg_ctx **out)
{
    if (!out) { set_error("out is NULL"); return DFTG_ERR_ARG; }
    *out = nullptr;
    if (!mol || !basis || !g || !mol->Z || !mol->xyz || !basis->bf_atom || !basis->bf_lmn || !basis->bf_nprim ||
        !basis->prim_alpha || !basis->prim_coef) {
        set_error("NULL argument");
        return DFTG_ERR_ARG;
    }
    if (mol->natoms < 1 || mol->natoms > kMaxAtoms) { set_error("natoms %d out of [1,%d]", mol->natoms, kMaxAtoms); return DFTG_ERR_ARG; }
    if (basis->nbf < 1) { set_error("nbf %d < 1", basis->nbf); return DFTG_ERR_ARG; }
    if (g->radial_points < 8 || g->radial_points > 2000) { set_error("radial_points %d out of [8,2000]", g->radial_points); return DFTG_ERR_ARG; }
    if (g->lebedev_order < 0 || g->lebedev_order >= DFTG_NUM_LEBEDEV_ORDERS) { set_error("lebedev_order %d out of [0,%d]", g->lebedev_order, DFTG_NUM_LEBEDEV_ORDERS - 1); return DFTG_ERR_ARG; }
    if (g->lmax < 0 || g->lmax > kLmaxCap) { set_error("lmax %d out of [0,%d]", g->lmax, kLmaxCap); return DFTG_ERR_ARG; }
    for (int a = 0; a < mol->natoms; ++a) {
        if (mol->Z[a] < 1 || mol->Z[a] > 18) { set_error("Z[%d] = %d out of [1,18]", a, mol->Z[a]); return DFTG_ERR_ARG; }
        for (int d = 0; d < 3; ++d)
            if (!std::isfinite(mol->xyz[3 * a + d])) { set_error("atom %d coordinate not finite", a); return DFTG_ERR_NONFINITE; }
        for (int b = 0; b < a; ++b) {
            double dx = mol->xyz[3 * a] - mol->xyz[3 * b], dy = mol->xyz[3 * a + 1] - mol->xyz[3 * b + 1],
                   dz = mol->xyz[3 * a + 2] - mol->xyz[3 * b + 2];
            if (dx * dx + dy * dy + dz * dz < 1e-12) { set_error("atoms %d and %d coincide", b, a); return DFTG_ERR_ARG; }
        }
    }
    long long np = 0;
    for (int i = 0; i < basis->nbf; ++i) {
        if (basis->bf_atom[i] < 0 || basis->bf_atom[i] >= mol->natoms) { set_error("bf_atom[%d] out of range", i); return DFTG_ERR_ARG; }
        if (basis->bf_nprim[i] < 1) { set_error("bf_nprim[%d] < 1", i); return DFTG_ERR_ARG; }
        int L = 0;
        for (int d = 0; d < 3; ++d) {
            if (basis->bf_lmn[3 * i + d] < 0) { set_error("bf_lmn[%d] negative", i); return DFTG_ERR_ARG; }
            L += basis->bf_lmn[3 * i + d];
        }
        if (L > 4) { set_error("bf %d: angular momentum %d > 4", i, L); return DFTG_ERR_ARG; }
        np += basis->bf_nprim[i];
    }
    for (long long k = 0; k < np; ++k)
        if (!(basis->prim_alpha[k] > 0.0) || !std::isfinite(basis->prim_coef[k])) {
            set_error("primitive %lld: bad exponent or coefficient", k);
            return DFTG_ERR_ARG;
        }
    dftg_ctx *c = new (std::nothrow) dftg_ctx();
    if (!c) { set_error("host allocation failed"); return DFTG_ERR_NOMEM; }
    int rc = build_ctx(c, mol, basis, g, cell0, ncell);
    if (rc != DFTG_OK) { free_ctx(c); return rc; }
    *out = c;
    return DFTG_OK;
}

// Context over explicit points (no atoms, cells or Hartree step): the
// amplitudes, the density, the LDA point kernel and the XC contraction of a
// synthetic contraction workload.  centres give the function centres (their
// Z are ignored).
static int build_points_ctx(dftg_ctx *c, const dftg_points *pts, const dftg_molecule *ctr, const dftg_basis *basis,
                            int device)
{
    c->device = device;
    c->points_only = true;
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    c->stream = c->own_stream;
    c->natoms = ctr->natoms;
    c->Z.assign(ctr->natoms, 0);
    c->xyz.assign(ctr->xyz, ctr->xyz + 3 * ctr->natoms);
    c->nbf = basis->nbf;
    c->bf_atom.assign(basis->bf_atom, basis->bf_atom + c->nbf);
    c->bf_lmn.assign(basis->bf_lmn, basis->bf_lmn + 3 * c->nbf);
    c->bf_off.assign(c->nbf + 1, 0);
    for (int i = 0; i < c->nbf; ++i) c->bf_off[i + 1] = c->bf_off[i] + basis->bf_nprim[i];
    c->nprim = c->bf_off[c->nbf];
    c->alpha.assign(basis->prim_alpha, basis->prim_alpha + c->nprim);
    c->coef.assign(basis->prim_coef, basis->prim_coef + c->nprim);
    c->norm.resize(c->nprim);
    std::vector<double> pcn(c->nprim);
    for (int i = 0; i < c->nbf; ++i)
        for (int k = c->bf_off[i]; k < c->bf_off[i + 1]; ++k) {
            c->norm[k] = gto_norm(c->alpha[k], c->bf_lmn[3 * i], c->bf_lmn[3 * i + 1], c->bf_lmn[3 * i + 2]);
            pcn[k] = c->coef[k] * c->norm[k];
        }
    c->nrad = 1;
    c->leb = 0;
    c->nang = 1;
    c->lmax = 0;
    c->nlm = 1;
    c->npts = pts->npts;
    c->npad = (c->npts + kPtsAlign - 1) / kPtsAlign * kPtsAlign;
    const size_t np = c->npad, nn = (size_t)c->nbf * c->nbf;
    DFTG_TRY(dalloc(&c->d_atoms, 4 * (size_t)c->natoms));
    DFTG_TRY(dalloc(&c->d_bf_lmn, 3 * (size_t)c->nbf));
    DFTG_TRY(dalloc(&c->d_bf_off, (size_t)c->nbf + 1));
    DFTG_TRY(dalloc(&c->d_bf_atom, (size_t)c->nbf));
    DFTG_TRY(dalloc(&c->d_pa, (size_t)c->nprim));
    DFTG_TRY(dalloc(&c->d_pcn, (size_t)c->nprim));
    DFTG_TRY(dalloc(&c->d_x, np));
    DFTG_TRY(dalloc(&c->d_y, np));
    DFTG_TRY(dalloc(&c->d_z, np));
    DFTG_TRY(dalloc(&c->d_w, np));
    DFTG_TRY(dalloc(&c->d_wb, np));
    DFTG_TRY(dalloc(&c->d_rho, np));
    DFTG_CUDA(cudaMalloc(&c->d_rw32, sizeof(float) * 2 * np));
    DFTG_CUDA(cudaMalloc(&c->d_wsplit, sizeof(float) * 4 * np));
    DFTG_TRY(dalloc(&c->d_V, np));
    DFTG_TRY(dalloc(&c->d_cxc, np));
    DFTG_TRY(dalloc(&c->d_cj, np));
    DFTG_TRY(dalloc(&c->d_cxc32, np));
    DFTG_TRY(dalloc(&c->d_cj32, np));
    DFTG_TRY(dalloc(&c->d_phi, np * c->nbf));
    DFTG_TRY(dalloc(&c->d_phi32, np * c->nbf));
    DFTG_TRY(dalloc(&c->d_P, nn));
    DFTG_TRY(dalloc(&c->d_P32, 2 * (size_t)c->nbf * ((c->nbf + 3) / 4 * 4)));   // FP32 hi, lo of P, rows padded to 4
    DFTG_TRY(dalloc(&c->d_J, nn));
    DFTG_TRY(dalloc(&c->d_XC, nn));
    int nsm = 0;
    DFTG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    size_t part = contract_part_elems(c->nbf, c->npad);
    const size_t part_tc = contract_tc_part_elems(c->nbf, c->npad, nsm);
    c->part_elems = part > part_tc ? part : part_tc;
    DFTG_TRY(dalloc(&c->d_part, c->part_elems));
    c->red_lda_off = reduction_elems(c->npad, 1, 1, (int)std::min<size_t>(c->npts, 0x7fffffff)) + 64;
    c->red_elems = c->red_lda_off + 2 * lda_blocks(c->npad);
    DFTG_TRY(dalloc(&c->d_red, c->red_elems));
    DFTG_TRY(dalloc(&c->d_scal, scal_elems(c->natoms)));
    DFTG_CUDA(cudaMalloc(&c->d_counters, sizeof(int) * kNumCounters));
    DFTG_CUDA(cudaMemset(c->d_counters, 0, sizeof(int) * kNumCounters));
    DFTG_CUDA(cudaMallocHost(&c->h_scal, sizeof(double) * (scal_elems(c->natoms) + 1)));   // + the wait flag
    DFTG_CUDA(cudaMemset(c->d_scal, 0, sizeof(double) * scal_elems(c->natoms)));
    std::vector<double> atoms(4 * (size_t)c->natoms, 0.0);
    for (int a = 0; a < c->natoms; ++a)
        for (int d = 0; d < 3; ++d) atoms[4 * a + d] = c->xyz[3 * a + d];
    // points as structure of arrays, padding at zero weight; w_becke = 1
    std::vector<double> X(np, 0.0), Y(np, 0.0), Zc(np, 0.0), W(np, 0.0), WB(np, 0.0);
    for (size_t p = 0; p < c->npts; ++p) {
        X[p] = pts->xyz[3 * p];
        Y[p] = pts->xyz[3 * p + 1];
        Zc[p] = pts->xyz[3 * p + 2];
        W[p] = pts->w[p];
        WB[p] = 1.0;
    }
    DFTG_CUDA(cudaMemcpy(c->d_atoms, atoms.data(), sizeof(double) * atoms.size(), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_x, X.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_y, Y.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_z, Zc.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_w, W.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_wb, WB.data(), sizeof(double) * np, cudaMemcpyHostToDevice));
    DFTG_TRY(launch_weight_planes(c));
    DFTG_CUDA(cudaMemset(c->d_cj, 0, sizeof(double) * np));
    DFTG_CUDA(cudaMemset(c->d_cj32, 0, sizeof(float) * np));
    DFTG_CUDA(cudaMemcpy(c->d_bf_lmn, c->bf_lmn.data(), sizeof(int) * 3 * c->nbf, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_bf_off, c->bf_off.data(), sizeof(int) * (c->nbf + 1), cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_bf_atom, c->bf_atom.data(), sizeof(int) * c->nbf, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_pa, c->alpha.data(), sizeof(double) * c->nprim, cudaMemcpyHostToDevice));
    DFTG_CUDA(cudaMemcpy(c->d_pcn, pcn.data(), sizeof(double) * c->nprim, cudaMemcpyHostToDevice));
    DFTG_TRY(launch_amplitudes(c));
    DFTG_TRY(contract_setup(c));
    DFTG_TRY(contract_tc_setup(c));
    DFTG_TRY(contract_tt_setup(c));
    DFTG_TRY(density_tc_setup(c));
    DFTG_TRY(density_tt_setup(c));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    return DFTG_OK;
}

int dftg_create_points(const dftg_points *pts, const dftg_molecule *centres, const dftg_basis *basis, int device,
                       dftg_ctx **out)
{
    if (!out) { set_error("out is NULL"); return DFTG_ERR_ARG; }
    *out = nullptr;
    if (!pts || !centres || !basis || !pts->xyz || !pts->w || !centres->xyz || !basis->bf_atom || !basis->bf_lmn ||
        !basis->bf_nprim || !basis->prim_alpha || !basis->prim_coef) {
        set_error("NULL argument");
        return DFTG_ERR_ARG;
    }
    if (pts->npts < 1) { set_error("npts 0"); return DFTG_ERR_ARG; }
    if (centres->natoms < 1) { set_error("no centres"); return DFTG_ERR_ARG; }
    if (basis->nbf < 1) { set_error("nbf %d < 1", basis->nbf); return DFTG_ERR_ARG; }
    for (size_t p = 0; p < pts->npts; ++p) {
        if (!std::isfinite(pts->xyz[3 * p]) || !std::isfinite(pts->xyz[3 * p + 1]) || !std::isfinite(pts->xyz[3 * p + 2]) ||
            !std::isfinite(pts->w[p])) {
            set_error("point %zu not finite", p);
            return DFTG_ERR_NONFINITE;
        }
    }
    for (int a = 0; a < 3 * centres->natoms; ++a)
        if (!std::isfinite(centres->xyz[a])) { set_error("centre coordinate not finite"); return DFTG_ERR_NONFINITE; }
    long long np = 0;
    for (int i = 0; i < basis->nbf; ++i) {
        if (basis->bf_atom[i] < 0 || basis->bf_atom[i] >= centres->natoms) { set_error("bf_atom[%d] out of range", i); return DFTG_ERR_ARG; }
        if (basis->bf_nprim[i] < 1) { set_error("bf_nprim[%d] < 1", i); return DFTG_ERR_ARG; }
        int L = 0;
        for (int d = 0; d < 3; ++d) {
            if (basis->bf_lmn[3 * i + d] < 0) { set_error("bf_lmn[%d] negative", i); return DFTG_ERR_ARG; }
            L += basis->bf_lmn[3 * i + d];
        }
        if (L > 4) { set_error("bf %d: angular momentum %d > 4", i, L); return DFTG_ERR_ARG; }
        np += basis->bf_nprim[i];
    }
    for (long long k = 0; k < np; ++k)
        if (!(basis->prim_alpha[k] > 0.0) || !std::isfinite(basis->prim_coef[k])) {
            set_error("primitive %lld: bad exponent or coefficient", k);
            return DFTG_ERR_ARG;
        }
    dftg_ctx *c = new (std::nothrow) dftg_ctx();
    if (!c) { set_error("host allocation failed"); return DFTG_ERR_NOMEM; }
    int rc = build_points_ctx(c, pts, centres, basis, device);
    if (rc != DFTG_OK) { free_ctx(c); return rc; }
    *out = c;
    return DFTG_OK;
}

// rho (no density correction), LDA point kernel, XC contraction; the scalars
// E_xc and the integrated density stay on the device
static int xc_pipeline(dftg_ctx *c)
{
    DFTG_TRY(launch_density(c));
    DFTG_TRY(launch_atom_sums(c, kSumsOnly));
    c->rho_scaled = false;
    DFTG_TRY(launch_xc_points(c, false));
    DFTG_TRY(launch_contract(c, true, false));
    return DFTG_OK;
}

int dftg_xc_build_device(dftg_ctx *c, const double *P_dev, double *XC_dev, double *scalars_dev)
{
    CHECK_CTX(c);
    if (!P_dev) { set_error("P_dev NULL"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    if (P_dev != c->d_P) DFTG_CUDA(cudaMemcpyAsync(c->d_P, P_dev, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    DFTG_TRY(xc_pipeline(c));
    if (XC_dev) DFTG_CUDA(cudaMemcpyAsync(XC_dev, c->d_XC, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    if (scalars_dev) {
        DFTG_CUDA(cudaMemcpyAsync(scalars_dev, c->d_scal + kScalExc, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        DFTG_CUDA(cudaMemcpyAsync(scalars_dev + 1, c->d_scal + kScalNelec, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
    c->have_density = true;
    c->have_hartree = false;
    c->have_build = false;
    return DFTG_OK;
}

int dftg_xc_build(dftg_ctx *c, const double *P, double *XC, double *exc, double *nelec)
{
    CHECK_CTX(c);
    if (!P) { set_error("P NULL"); return DFTG_ERR_ARG; }
    DFTG_TRY(check_matrix(P, c->nbf));
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    DFTG_CUDA(cudaMemcpyAsync(c->d_P, P, sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream));
    DFTG_TRY(xc_pipeline(c));
    if (XC) DFTG_CUDA(cudaMemcpyAsync(XC, c->d_XC, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    DFTG_TRY(sync_scalars(c));
    if (exc) *exc = c->h_scal[kScalExc];
    if (nelec) *nelec = c->h_scal[kScalNelec];
    c->have_density = true;
    c->have_hartree = false;
    c->have_build = false;
    return DFTG_OK;
}

int dftg_destroy(dftg_ctx *c)
{
    free_ctx(c);
    return DFTG_OK;
}

int dftg_grid_size(const dftg_ctx *c, size_t *npts)
{
    CHECK_CTX(c);
    if (!npts) { set_error("npts NULL"); return DFTG_ERR_ARG; }
    *npts = c->npts;
    return DFTG_OK;
}

int dftg_nbf(const dftg_ctx *c, int *nbf)
{
    CHECK_CTX(c);
    if (!nbf) { set_error("nbf NULL"); return DFTG_ERR_ARG; }
    *nbf = c->nbf;
    return DFTG_OK;
}

int dftg_set_precision(dftg_ctx *c, int precision)
{
    CHECK_CTX(c);
    if (precision != DFTG_PREC_FP64 && precision != DFTG_PREC_MIXED) { set_error("unknown precision %d", precision); return DFTG_ERR_ARG; }
    c->precision = precision;
    c->prec_mask = precision == DFTG_PREC_MIXED ? (unsigned)kPrecAll : 0u;
    return DFTG_OK;
}

int dftg_set_precision_mask(dftg_ctx *c, unsigned mask)
{
    CHECK_CTX(c);
    if (mask & ~(unsigned)kPrecAll) { set_error("unknown precision bits 0x%x", mask); return DFTG_ERR_ARG; }
    c->prec_mask = mask;
    c->precision = mask ? DFTG_PREC_MIXED : DFTG_PREC_FP64;
    return DFTG_OK;
}

int dftg_set_stream(dftg_ctx *c, void *s)
{
    CHECK_CTX(c);
    if (s == reinterpret_cast<void *>(cudaStreamLegacy) || s == reinterpret_cast<void *>(cudaStreamPerThread)) {
        set_error("the default streams cannot be captured into the build's CUDA graph: pass a created stream");
        return DFTG_ERR_ARG;
    }
    c->stream = s ? reinterpret_cast<cudaStream_t>(s) : c->own_stream;
    return DFTG_OK;
}

int dftg_set_density(dftg_ctx *c, const double *P)
{
    CHECK_CTX(c);
    if (!P) { set_error("P NULL"); return DFTG_ERR_ARG; }
    DFTG_TRY(check_matrix(P, c->nbf));
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_CUDA(cudaMemcpyAsync(c->d_P, P, sizeof(double) * c->nbf * c->nbf, cudaMemcpyHostToDevice, c->stream));
    DFTG_TRY(launch_density(c));
    DFTG_TRY(launch_atom_sums(c, kSumsOnly));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    c->have_density = true;
    c->have_hartree = false;
    c->rho_scaled = false;
    c->have_build = false;
    return DFTG_OK;
}

int dftg_correct_densities(dftg_ctx *c, double *scale)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (c->points_only) { set_error("a point-set context has no atoms: no Hartree step or density correction"); return DFTG_ERR_STATE; }
    if (!c->have_density) { set_error("correct_densities before set_density"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY(launch_atom_sums(c, kSumsCorrect));
    c->rho_scaled = true;
    DFTG_TRY(sync_scalars(c));
    if (scale) *scale = c->h_scal[kScalScale];
    return DFTG_OK;
}

int dftg_calculate_density(dftg_ctx *c, double *nelec)
{
    CHECK_CTX(c);
    if (!nelec) { set_error("nelec NULL"); return DFTG_ERR_ARG; }
    if (!c->have_density) { set_error("calculate_density before set_density"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY(launch_atom_sums(c, kSumsOnly));
    DFTG_TRY(sync_scalars(c));
    *nelec = c->h_scal[kScalNelec];
    return DFTG_OK;
}

int dftg_calculate_hartree_potential(dftg_ctx *c, double *J)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (c->points_only) { set_error("a point-set context has no atoms: no Hartree step or density correction"); return DFTG_ERR_STATE; }
    if (!c->have_density) { set_error("calculate_hartree_potential before set_density"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY(launch_atom_sums(c, kSumsOnly));   // per-atom charges of the current rho
    DFTG_TRY(launch_hartree(c));
    DFTG_TRY(launch_contract(c, false, true));
    if (J) DFTG_CUDA(cudaMemcpyAsync(J, c->d_J, sizeof(double) * c->nbf * c->nbf, cudaMemcpyDeviceToHost, c->stream));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    c->have_hartree = true;
    return DFTG_OK;
}

int dftg_calculate_xc(dftg_ctx *c, double *XC, double *exc)
{
    CHECK_CTX(c);
    if (!c->have_density) { set_error("calculate_xc before set_density"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY(launch_xc_points(c, false));
    DFTG_TRY(launch_contract(c, true, false));
    if (XC) DFTG_CUDA(cudaMemcpyAsync(XC, c->d_XC, sizeof(double) * c->nbf * c->nbf, cudaMemcpyDeviceToHost, c->stream));
    DFTG_TRY(sync_scalars(c));
    if (exc) *exc = c->h_scal[kScalExc];
    return DFTG_OK;
}

int dftg_fock_build_device(dftg_ctx *c, const double *P_dev, double *J_dev, double *XC_dev, double *scalars_dev)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (c->points_only) { set_error("a point-set context has no atoms: no Hartree step or density correction"); return DFTG_ERR_STATE; }
    if (!P_dev) { set_error("P_dev NULL"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    if (P_dev != c->d_P) DFTG_CUDA(cudaMemcpyAsync(c->d_P, P_dev, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    DFTG_TRY(fock_pipeline_graph(c));
    if (J_dev) DFTG_CUDA(cudaMemcpyAsync(J_dev, c->d_J, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    if (XC_dev) DFTG_CUDA(cudaMemcpyAsync(XC_dev, c->d_XC, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    if (scalars_dev) {
        DFTG_CUDA(cudaMemcpyAsync(scalars_dev, c->d_scal + kScalExc, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        DFTG_CUDA(cudaMemcpyAsync(scalars_dev + 1, c->d_scal + kScalNelec, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        DFTG_CUDA(cudaMemcpyAsync(scalars_dev + 2, c->d_scal + kScalEJ, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
    c->have_density = true;
    c->have_hartree = true;
    c->have_build = true;
    c->fwd_mask = c->prec_mask;
    return DFTG_OK;
}

int dftg_fock_build_profile(dftg_ctx *c, const double *P_dev, double *phase_ms, const char **names, int cap,
                            int *nphase)
{
    CHECK_CTX(c);
    if (!c->points_only) CHECK_WHOLE(c);
    if (!P_dev || !phase_ms || !nphase) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    c->prof_n = 0;
    c->prof_on = true;
    int rc = mark(c, "start");
    if (rc == DFTG_OK && P_dev != c->d_P) {
        cudaError_t e = cudaMemcpyAsync(c->d_P, P_dev, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream);
        if (e != cudaSuccess) rc = cuda_fail(e, "copy P", __FILE__, __LINE__);
    }
    if (rc == DFTG_OK) rc = c->points_only ? xc_pipeline(c) : fock_pipeline(c);
    c->prof_on = false;
    if (rc != DFTG_OK) return rc;
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    const int n = c->prof_n - 1 < cap ? c->prof_n - 1 : cap;
    for (int i = 0; i < n; ++i) {
        float ms = 0.f;
        DFTG_CUDA(cudaEventElapsedTime(&ms, c->prof_ev[i], c->prof_ev[i + 1]));
        phase_ms[i] = ms;
        if (names) names[i] = c->prof_name[i + 1];
    }
    *nphase = n;
    c->have_density = true;
    c->have_hartree = !c->points_only;
    c->have_build = !c->points_only;
    if (!c->points_only) c->fwd_mask = c->prec_mask;
    return DFTG_OK;
}

int dftg_fock_build(dftg_ctx *c, const double *P, double *J, double *XC, double *exc, double *nelec)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (c->points_only) { set_error("a point-set context has no atoms: no Hartree step or density correction"); return DFTG_ERR_STATE; }
    if (!P) { set_error("P NULL"); return DFTG_ERR_ARG; }
    DFTG_TRY(check_matrix(P, c->nbf));
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    DFTG_CUDA(cudaMemcpyAsync(c->d_P, P, sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream));
    DFTG_TRY(fock_pipeline_graph(c));
    if (J) DFTG_CUDA(cudaMemcpyAsync(J, c->d_J, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    if (XC) DFTG_CUDA(cudaMemcpyAsync(XC, c->d_XC, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    DFTG_TRY(sync_scalars(c));
    if (exc) *exc = c->h_scal[kScalExc];
    if (nelec) *nelec = c->h_scal[kScalNelec];
    c->have_density = true;
    c->have_hartree = true;
    c->have_build = true;
    c->fwd_mask = c->prec_mask;
    return DFTG_OK;
}

// ------------------------------------------------------------------ atom-cell shards
// A build split by fuzzy cell over the contexts of a partition (one per rank),
// with three exchanges between the calls: the sum of w rho, every cell's
// spline data, and J, XC and the energies (moleculargrid.cpp:132-146, 336-389).
static int shard_check(dftg_ctx *c, int phase)
{
    CHECK_CTX(c);
    if (c->points_only) { set_error("a point-set context has no cells"); return DFTG_ERR_STATE; }
    if (c->shard_phase < phase) { set_error("shard call out of order (phase %d before %d)", phase, c->shard_phase + 1); return DFTG_ERR_STATE; }
    return DFTG_OK;
}

size_t shard_blob_doubles(const dftg_ctx *c)
{
    // FP64 spline coefficients [nlm][nrad][4], then the split FP32 table [nlm][nrad][8]
    return (size_t)c->nlm * c->nrad * 4 + (size_t)c->nlm * c->nrad * 4;
}

int dftg_shard_blob_size(const dftg_ctx *c, size_t *doubles_per_cell, int *first_cell, int *ncells)
{
    CHECK_CTX(c);
    if (c->points_only) { set_error("a point-set context has no cells"); return DFTG_ERR_STATE; }
    if (doubles_per_cell) *doubles_per_cell = shard_blob_doubles(c);
    if (first_cell) *first_cell = c->cell0;
    if (ncells) *ncells = c->ncell;
    return DFTG_OK;
}

int dftg_shard_density(dftg_ctx *c, const double *P, double *sum_wrho)
{
    DFTG_TRY(shard_check(c, 0));
    if (!P || !sum_wrho) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    DFTG_TRY(check_matrix(P, c->nbf));
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t nn = (size_t)c->nbf * c->nbf;
    DFTG_CUDA(cudaMemcpyAsync(c->d_P, P, sizeof(double) * nn, cudaMemcpyHostToDevice, c->stream));
    DFTG_TRY(launch_density(c));
    DFTG_TRY(launch_atom_sums(c, kSumsOnly));   // per cell: kScalAtomQ + local index; total in kScalNelec
    DFTG_TRY(sync_scalars(c));
    *sum_wrho = c->h_scal[kScalNelec];
    c->rho_scaled = false;
    c->have_build = false;
    c->shard_phase = 1;
    return DFTG_OK;
}

int dftg_shard_multipoles(dftg_ctx *c, double total_wrho, double *blob, size_t cap)
{
    DFTG_TRY(shard_check(c, 1));
    const size_t per = shard_blob_doubles(c);
    if (!blob || cap < per * c->ncell) { set_error("blob capacity %zu < %zu", cap, per * c->ncell); return DFTG_ERR_ARG; }
    if (!(total_wrho > 0.0) || !std::isfinite(total_wrho)) { set_error("total %g is not a positive number", total_wrho); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    // correction factor over the whole molecule (every atom's charge), charges of
    // this context's cells at their atoms' slots
    double charge = 0.0;
    for (int a = 0; a < c->natoms; ++a) charge += (double)c->Z[a];
    const double cf = charge / total_wrho;
    const size_t ns = scal_elems(c->natoms);
    std::vector<double> sc(c->h_scal, c->h_scal + ns);
    std::vector<double> raw(c->h_scal + kScalAtomQ, c->h_scal + kScalAtomQ + c->ncell);
    double n = 0.0;
    for (int t = 0; t < c->ncell; ++t) {
        sc[kScalAtomQ + c->cell0 + t] = raw[t] * cf;
        n += raw[t] * cf;
    }
    sc[kScalSum] = total_wrho;
    sc[kScalScale] = cf;
    sc[kScalNelec] = n;
    std::copy(sc.begin(), sc.end(), c->h_scal);
    DFTG_CUDA(cudaMemcpyAsync(c->d_scal, c->h_scal, sizeof(double) * ns, cudaMemcpyHostToDevice, c->stream));
    DFTG_TRY(launch_xc_points(c, true));        // rho *= cf, point kernel, this shard's E_xc
    c->rho_scaled = true;
    DFTG_TRY(launch_hartree_multipoles(c));
    const size_t n4 = (size_t)c->nlm * c->nrad * 4, n8 = (size_t)c->nlm * c->nrad * 8;
    DFTG_CUDA(cudaMemcpy2DAsync(blob, sizeof(double) * per, c->d_spl + (size_t)c->cell0 * n4, sizeof(double) * n4,
                                sizeof(double) * n4, (size_t)c->ncell, cudaMemcpyDeviceToHost, c->stream));
    DFTG_CUDA(cudaMemcpy2DAsync(blob + n4, sizeof(double) * per, c->d_splm + (size_t)c->cell0 * n8, sizeof(float) * n8,
                                sizeof(float) * n8, (size_t)c->ncell, cudaMemcpyDeviceToHost, c->stream));
    DFTG_TRY(sync_scalars(c));
    c->shard_phase = 2;
    return DFTG_OK;
}

int dftg_shard_finish(dftg_ctx *c, const double *blob_all, size_t cap, double *J, double *XC, double *scalars)
{
    DFTG_TRY(shard_check(c, 2));
    const size_t per = shard_blob_doubles(c);
    if (!blob_all || cap < per * c->natoms) { set_error("blob capacity %zu < %zu", cap, per * c->natoms); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    const size_t n4 = (size_t)c->nlm * c->nrad * 4, n8 = (size_t)c->nlm * c->nrad * 8;
    DFTG_CUDA(cudaMemcpy2DAsync(c->d_spl, sizeof(double) * n4, blob_all, sizeof(double) * per, sizeof(double) * n4,
                                (size_t)c->natoms, cudaMemcpyHostToDevice, c->stream));
    DFTG_CUDA(cudaMemcpy2DAsync(c->d_splm, sizeof(float) * n8, blob_all + n4, sizeof(double) * per, sizeof(float) * n8,
                                (size_t)c->natoms, cudaMemcpyHostToDevice, c->stream));
    DFTG_TRY(launch_hartree_cross(c));
    DFTG_TRY(launch_contract(c, true, true));
    const size_t nn = (size_t)c->nbf * c->nbf;
    if (J) DFTG_CUDA(cudaMemcpyAsync(J, c->d_J, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    if (XC) DFTG_CUDA(cudaMemcpyAsync(XC, c->d_XC, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    DFTG_TRY(sync_scalars(c));
    if (scalars) {
        scalars[0] = c->h_scal[kScalExc];
        scalars[1] = c->h_scal[kScalNelec];
        scalars[2] = c->h_scal[kScalEJ];
    }
    c->have_density = true;
    c->have_hartree = true;
    c->shard_phase = 0;
    return DFTG_OK;
}

static int get_points(const dftg_ctx *c, const double *src, double *out, size_t cap, size_t mult)
{
    CHECK_CTX(c);
    if (!out) { set_error("out NULL"); return DFTG_ERR_ARG; }
    if (cap < c->npts * mult) { set_error("capacity %zu < %zu", cap, c->npts * mult); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    DFTG_CUDA(cudaMemcpy(out, src, sizeof(double) * c->npts, cudaMemcpyDeviceToHost));
    return DFTG_OK;
}

int dftg_get_weights(const dftg_ctx *c, double *out, size_t cap) { return get_points(c, c ? c->d_w : nullptr, out, cap, 1); }
int dftg_get_becke_weights(const dftg_ctx *c, double *out, size_t cap) { return get_points(c, c ? c->d_wb : nullptr, out, cap, 1); }
int dftg_get_densities(const dftg_ctx *c, double *out, size_t cap) { return get_points(c, c ? c->d_rho : nullptr, out, cap, 1); }
int dftg_get_potential(const dftg_ctx *c, double *out, size_t cap) { return get_points(c, c ? c->d_V : nullptr, out, cap, 1); }

int dftg_get_positions(const dftg_ctx *c, double *out, size_t cap)
{
    CHECK_CTX(c);
    if (!out) { set_error("out NULL"); return DFTG_ERR_ARG; }
    if (cap < 3 * c->npts) { set_error("capacity %zu < %zu", cap, 3 * c->npts); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<double> t(c->npts);
    const double *src[3] = {c->d_x, c->d_y, c->d_z};
    for (int d = 0; d < 3; ++d) {
        DFTG_CUDA(cudaMemcpy(t.data(), src[d], sizeof(double) * c->npts, cudaMemcpyDeviceToHost));
        for (size_t p = 0; p < c->npts; ++p) out[3 * p + d] = t[p];
    }
    return DFTG_OK;
}

int dftg_get_amplitudes(const dftg_ctx *c, double *out, size_t cap)
{
    CHECK_CTX(c);
    if (!out) { set_error("out NULL"); return DFTG_ERR_ARG; }
    const size_t need = c->npts * (size_t)c->nbf;
    if (cap < need) { set_error("capacity %zu < %zu", cap, need); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    std::vector<double> t(c->npts);
    for (int mu = 0; mu < c->nbf; ++mu) {
        DFTG_CUDA(cudaMemcpy(t.data(), c->d_phi + (size_t)mu * c->npad, sizeof(double) * c->npts, cudaMemcpyDeviceToHost));
        for (size_t p = 0; p < c->npts; ++p) out[mu + p * (size_t)c->nbf] = t[p];
    }
    return DFTG_OK;
}

int dftg_get_energies(dftg_ctx *c, double *exc, double *ej, double *nelec)
{
    CHECK_CTX(c);
    DFTG_CUDA(cudaSetDevice(c->device));
    DFTG_TRY(sync_scalars(c));
    if (exc) *exc = c->h_scal[kScalExc];
    if (ej) *ej = c->h_scal[kScalEJ];
    if (nelec) *nelec = c->h_scal[kScalNelec];
    return DFTG_OK;
}

int dftg_backward_device(dftg_ctx *c, double seed_exc, double seed_ej, double *dEdP_dev, double *dEdR_dev)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (!c->have_build) { set_error("backward before a complete Fock build"); return DFTG_ERR_STATE; }
    if (!std::isfinite(seed_exc) || !std::isfinite(seed_ej)) { set_error("non-finite seed"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    return launch_backward(c, seed_exc, seed_ej, dEdP_dev, dEdR_dev);
}

int dftg_backward(dftg_ctx *c, double seed_exc, double seed_ej, double *dEdP, double *dEdR)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (!c->have_build) { set_error("backward before a complete Fock build"); return DFTG_ERR_STATE; }
    if (!std::isfinite(seed_exc) || !std::isfinite(seed_ej)) { set_error("non-finite seed"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(c->device));
    if (!c->d_bw_out) {
        DFTG_CUDA(cudaMalloc(&c->d_bw_out, sizeof(double) * ((size_t)c->nbf * c->nbf + (size_t)c->natoms * 3)));
    }
    const size_t nn = (size_t)c->nbf * c->nbf;
    double *dP = dEdP ? c->d_bw_out : nullptr, *dR = dEdR ? c->d_bw_out + nn : nullptr;
    DFTG_TRY(launch_backward(c, seed_exc, seed_ej, dP, dR));
    if (dEdP) DFTG_CUDA(cudaMemcpyAsync(dEdP, dP, sizeof(double) * nn, cudaMemcpyDeviceToHost, c->stream));
    if (dEdR) DFTG_CUDA(cudaMemcpyAsync(dEdR, dR, sizeof(double) * 3 * c->natoms, cudaMemcpyDeviceToHost, c->stream));
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    return DFTG_OK;
}

int dftg_backward_profile(dftg_ctx *c, double seed_exc, double seed_ej, double *phase_ms, const char **names,
                          int cap, int *nphase)
{
    CHECK_CTX(c);
    if (!phase_ms || !nphase) { set_error("NULL argument"); return DFTG_ERR_ARG; }
    if (!c->have_build) { set_error("backward before a complete Fock build"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    if (!c->d_bw_out)
        DFTG_CUDA(cudaMalloc(&c->d_bw_out, sizeof(double) * ((size_t)c->nbf * c->nbf + (size_t)c->natoms * 3)));
    c->prof_n = 0;
    c->prof_on = true;
    int rc = mark(c, "start");
    if (rc == DFTG_OK)
        rc = launch_backward(c, seed_exc, seed_ej, c->d_bw_out, c->d_bw_out + (size_t)c->nbf * c->nbf);
    c->prof_on = false;
    if (rc != DFTG_OK) return rc;
    DFTG_CUDA(cudaStreamSynchronize(c->stream));
    const int n = c->prof_n - 1 < cap ? c->prof_n - 1 : cap;
    for (int i = 0; i < n; ++i) {
        float ms = 0.f;
        DFTG_CUDA(cudaEventElapsedTime(&ms, c->prof_ev[i], c->prof_ev[i + 1]));
        phase_ms[i] = ms;
        if (names) names[i] = c->prof_name[i + 1];
    }
    *nphase = n;
    return DFTG_OK;
}

int dftg_get_launch_shape(const dftg_ctx *c, int *shape, int cap)
{
    CHECK_CTX(c);
    if (!shape || cap < 3) { set_error("shape needs 3 entries"); return DFTG_ERR_ARG; }
    shape[0] = c->tc_ready ? c->tc_grid : 0;
    shape[1] = c->ct_ready ? c->ct_grid : 0;
    shape[2] = c->ct_ready ? c->ct_nst : 0;
    return DFTG_OK;
}

int dftg_set_launch_shape(dftg_ctx *c, const int *shape, int n)
{
    CHECK_CTX(c);
    if (!shape || n < 3) { set_error("shape needs 3 entries"); return DFTG_ERR_ARG; }
    if (c->tc_ready) {
        if (shape[0] < 1 || shape[0] > c->tc_grid_max) { set_error("density CTAs %d outside 1..%d", shape[0], c->tc_grid_max); return DFTG_ERR_ARG; }
        c->tc_grid = shape[0];
    }
    if (c->ct_ready) {
        if (shape[1] < 1 || shape[1] > c->ct_grid_max) { set_error("contraction CTAs %d outside 1..%d", shape[1], c->ct_grid_max); return DFTG_ERR_ARG; }
        if (shape[2] < c->ct_nst_min || shape[2] > c->ct_nst_max || (shape[2] & 1)) {
            set_error("contraction stages %d: an even count in %d..%d", shape[2], c->ct_nst_min, c->ct_nst_max);
            return DFTG_ERR_ARG;
        }
        c->ct_grid = shape[1];
        c->ct_nst = shape[2];
    }
    return DFTG_OK;
}

// mean device time of reps graph-replayed builds on the context's own P
static int time_builds(dftg_ctx *c, int reps, double *ms)
{
    DFTG_TRY(fock_pipeline_graph(c));   // eager (new shape) or replay
    DFTG_TRY(fock_pipeline_graph(c));   // capture
    cudaEvent_t e0, e1;
    DFTG_CUDA(cudaEventCreate(&e0));
    DFTG_CUDA(cudaEventCreate(&e1));
    int rc = DFTG_OK;
    if (cudaEventRecord(e0, c->stream) != cudaSuccess) rc = DFTG_ERR_CUDA;
    for (int r = 0; r < reps && rc == DFTG_OK; ++r) rc = fock_pipeline_graph(c);
    if (rc == DFTG_OK && cudaEventRecord(e1, c->stream) != cudaSuccess) rc = DFTG_ERR_CUDA;
    float t = 0.f;
    if (rc == DFTG_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = DFTG_ERR_CUDA;
    if (rc == DFTG_OK && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) rc = DFTG_ERR_CUDA;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc != DFTG_OK) { set_error("autotune timing failed"); return rc; }
    DFTG_TRY(sync_scalars(c));          // a bounded device wait that expired fails the candidate
    *ms = (double)t / reps;
    return DFTG_OK;
}

static void shape_candidates(int mx, std::vector<int> &out)
{
    out.clear();
    const int f[5][2] = {{1, 1}, {3, 4}, {1, 2}, {1, 4}, {1, 8}};
    for (const auto &q : f) {
        const int v = mx * q[0] / q[1];
        if (v >= 1 && std::find(out.begin(), out.end(), v) == out.end()) out.push_back(v);
    }
}

int dftg_autotune(dftg_ctx *c, int reps, double *best_ms)
{
    CHECK_CTX(c);
    CHECK_WHOLE(c);
    if (reps < 1) { set_error("reps < 1"); return DFTG_ERR_ARG; }
    if (!c->have_build) { set_error("autotune before a complete Fock build (it times builds of that P)"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(c->device));
    double best = 0.0;
    DFTG_TRY(time_builds(c, reps, &best));
    const bool tune_tc = c->tc_ready && (c->prec_mask & kPrecDensity);
    const bool tune_ct = c->ct_ready && (c->prec_mask & kPrecContract);
    std::vector<int> cand;
    // coordinate descent over the three shapes, each from the current best
    for (int knob = 0; knob < 3; ++knob) {
        int *field = knob == 0 ? &c->tc_grid : (knob == 1 ? &c->ct_grid : &c->ct_nst);
        if ((knob == 0 && !tune_tc) || (knob > 0 && !tune_ct)) continue;
        if (knob == 2) {
            cand.clear();
            for (int v = c->ct_nst_max; v >= c->ct_nst_min; v -= 2) cand.push_back(v);   // even depths
        } else {
            shape_candidates(knob == 0 ? c->tc_grid_max : c->ct_grid_max, cand);
        }
        const int keep = *field;
        int best_v = keep;
        for (int v : cand) {
            if (v == keep) continue;
            *field = v;
            double t = 0.0;
            DFTG_TRY(time_builds(c, reps, &t));
            if (t < best) { best = t; best_v = v; }
        }
        *field = best_v;
    }
    DFTG_TRY(fock_pipeline_graph(c));   // leave the outputs of the chosen shape
    DFTG_TRY(sync_scalars(c));
    if (best_ms) *best_ms = best;
    return DFTG_OK;
}

int dftg_nuclear_repulsion(const dftg_ctx *c, double *enuc)
{
    CHECK_CTX(c);
    if (!enuc) { set_error("enuc NULL"); return DFTG_ERR_ARG; }
    double e = 0.0;   // dft.cpp:235-246
    for (int i = 0; i < c->natoms; ++i)
        for (int j = i + 1; j < c->natoms; ++j) {
            double dx = c->xyz[3 * i] - c->xyz[3 * j], dy = c->xyz[3 * i + 1] - c->xyz[3 * j + 1],
                   dz = c->xyz[3 * i + 2] - c->xyz[3 * j + 2];
            e += c->Z[i] * c->Z[j] / std::sqrt(dx * dx + dy * dy + dz * dz);
        }
    *enuc = e;
    return DFTG_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ batches

constexpr unsigned long long kBatchWaitNs = 2000000000ull;   // limit of the persistent launches' waits: 2 s

struct dftg_batch {
    std::vector<dftg_ctx *> ctx;
    std::vector<cudaEvent_t> join;      // per context: end of its branch (graph of branches)
    cudaEvent_t fork = nullptr;
    cudaGraphExec_t exec = nullptr;
    std::vector<const void *> key;      // buffers, masks, shapes, mode and stream the graph was captured with
    bool warm = false;
    int mode = DFTG_BATCH_PERSISTENT;
    dftg::BatchPlan *plan = nullptr;    // persistent launches: device records of the current key
    cudaStream_t last = nullptr;        // stream of the last launch
};

static void batch_free(dftg_batch *b)
{
    if (!b) return;
    if (b->last) cudaStreamSynchronize(b->last);
    dftg::batch_plan_free(b->plan);
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->fork) cudaEventDestroy(b->fork);
    for (cudaEvent_t e : b->join)
        if (e) cudaEventDestroy(e);
    delete b;
}

// one context's build on its own stream (copies in and out included)
static int batch_branch(dftg_ctx *c, const double *P, double *J, double *XC, double *sc)
{
    const size_t nn = (size_t)c->nbf * c->nbf;
    if (P != c->d_P) DFTG_CUDA(cudaMemcpyAsync(c->d_P, P, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    DFTG_TRY(fock_pipeline(c));
    if (J) DFTG_CUDA(cudaMemcpyAsync(J, c->d_J, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    if (XC) DFTG_CUDA(cudaMemcpyAsync(XC, c->d_XC, sizeof(double) * nn, cudaMemcpyDeviceToDevice, c->stream));
    if (sc) {
        DFTG_CUDA(cudaMemcpyAsync(sc, c->d_scal + kScalExc, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        DFTG_CUDA(cudaMemcpyAsync(sc + 1, c->d_scal + kScalNelec, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
        DFTG_CUDA(cudaMemcpyAsync(sc + 2, c->d_scal + kScalEJ, sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    }
    c->have_density = true;
    c->have_hartree = true;
    c->have_build = true;
    c->fwd_mask = c->prec_mask;
    return DFTG_OK;
}

extern "C" int dftg_batch_create(dftg_ctx *const *ctxs, int n, dftg_batch **out)
{
    if (!out) { set_error("out is NULL"); return DFTG_ERR_ARG; }
    *out = nullptr;
    if (!ctxs || n < 1) { set_error("empty batch"); return DFTG_ERR_ARG; }
    for (int i = 0; i < n; ++i) {
        if (!ctxs[i]) { set_error("context %d is NULL", i); return DFTG_ERR_ARG; }
        for (int j = 0; j < i; ++j)
            if (ctxs[j] == ctxs[i]) { set_error("context %d repeated", i); return DFTG_ERR_ARG; }
        if (ctxs[i]->device != ctxs[0]->device) { set_error("contexts on different devices"); return DFTG_ERR_ARG; }
        if (ctxs[i]->points_only) { set_error("context %d is a point-set context (no Fock build)", i); return DFTG_ERR_ARG; }
        if (ctxs[i]->cell0 != 0 || ctxs[i]->ncell != ctxs[i]->natoms) { set_error("context %d holds part of its molecule's cells", i); return DFTG_ERR_ARG; }
    }
    dftg_batch *b = new (std::nothrow) dftg_batch();
    if (!b) { set_error("host allocation failed"); return DFTG_ERR_NOMEM; }
    b->ctx.assign(ctxs, ctxs + n);
    b->join.assign(n, nullptr);
    cudaError_t e = cudaSetDevice(ctxs[0]->device);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
    for (int i = 0; i < n && e == cudaSuccess; ++i) e = cudaEventCreateWithFlags(&b->join[i], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        batch_free(b);
        return cuda_fail(e, "batch events", __FILE__, __LINE__);
    }
    *out = b;
    return DFTG_OK;
}

extern "C" int dftg_batch_destroy(dftg_batch *b)
{
    batch_free(b);
    return DFTG_OK;
}

extern "C" int dftg_batch_fock_build_device(dftg_batch *b, const double *const *P_devs, double *const *J_devs,
                                            double *const *XC_devs, double *const *scalars_devs, void *stream)
{
    if (!b) { set_error("null batch"); return DFTG_ERR_ARG; }
    if (!P_devs) { set_error("P_devs NULL"); return DFTG_ERR_ARG; }
    const int n = (int)b->ctx.size();
    for (int i = 0; i < n; ++i)
        if (!P_devs[i]) { set_error("P_devs[%d] NULL", i); return DFTG_ERR_ARG; }
    if (stream == reinterpret_cast<void *>(cudaStreamLegacy) || stream == reinterpret_cast<void *>(cudaStreamPerThread)) {
        set_error("the default streams cannot be captured into the batch's CUDA graph: pass a created stream");
        return DFTG_ERR_ARG;
    }
    DFTG_CUDA(cudaSetDevice(b->ctx[0]->device));
    cudaStream_t s0 = stream ? reinterpret_cast<cudaStream_t>(stream) : b->ctx[0]->stream;
    bool persist = b->mode == DFTG_BATCH_PERSISTENT;
    for (int i = 0; i < n && persist; ++i) persist = dftg::batch_group_eligible(b->ctx[i]);
    std::vector<const void *> key;
    key.push_back(s0);
    key.push_back(reinterpret_cast<const void *>((uintptr_t)(persist ? 1 : 0)));
    for (int i = 0; i < n; ++i) {
        key.push_back(P_devs[i]);
        key.push_back(J_devs ? J_devs[i] : nullptr);
        key.push_back(XC_devs ? XC_devs[i] : nullptr);
        key.push_back(scalars_devs ? scalars_devs[i] : nullptr);
        key.push_back(reinterpret_cast<const void *>((uintptr_t)b->ctx[i]->prec_mask));
        key.push_back(b->ctx[i]->stream);
        key.push_back(reinterpret_cast<const void *>((uintptr_t)b->ctx[i]->tc_grid));
        key.push_back(reinterpret_cast<const void *>((uintptr_t)b->ctx[i]->ct_grid));
        key.push_back(reinterpret_cast<const void *>((uintptr_t)b->ctx[i]->ct_nst));
    }
    if (key != b->key) {
        if (b->exec) cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
        b->warm = false;
        if (b->plan) {                  // its device records may still be read by a running batch
            if (b->last) DFTG_CUDA(cudaStreamSynchronize(b->last));
            dftg::batch_plan_free(b->plan);
            b->plan = nullptr;
        }
    }
    if (persist && !b->plan)
        DFTG_TRY(dftg::batch_plan_create(b->ctx.data(), n, P_devs, J_devs, XC_devs, scalars_devs, &b->plan));
    // the persistent launches run on s0 alone: s0 first waits for the work queued
    // on the contexts' own streams (set-up, earlier builds), and those streams
    // wait for the batch afterwards (outside any capture)
    auto order_before = [&]() -> int {
        if (!persist) return DFTG_OK;
        for (int i = 0; i < n; ++i)
            if (b->ctx[i]->stream != s0) {
                DFTG_CUDA(cudaEventRecord(b->join[i], b->ctx[i]->stream));
                DFTG_CUDA(cudaStreamWaitEvent(s0, b->join[i], 0));
            }
        return DFTG_OK;
    };
    auto order_after = [&]() -> int {
        if (!persist) return DFTG_OK;
        DFTG_CUDA(cudaEventRecord(b->fork, s0));
        for (dftg_ctx *c : b->ctx)
            if (c->stream != s0) DFTG_CUDA(cudaStreamWaitEvent(c->stream, b->fork, 0));
        return DFTG_OK;
    };
    auto enqueue = [&]() -> int {
        if (persist) return dftg::batch_plan_enqueue(b->plan, s0, -1, kBatchWaitNs, false);
        // fork: every branch waits for s0, s0 waits for every branch
        DFTG_CUDA(cudaEventRecord(b->fork, s0));
        for (int i = 0; i < n; ++i) {
            dftg_ctx *c = b->ctx[i];
            if (c->stream != s0) DFTG_CUDA(cudaStreamWaitEvent(c->stream, b->fork, 0));
            DFTG_TRY(batch_branch(c, P_devs[i], J_devs ? J_devs[i] : nullptr, XC_devs ? XC_devs[i] : nullptr,
                                  scalars_devs ? scalars_devs[i] : nullptr));
            if (c->stream != s0) {
                DFTG_CUDA(cudaEventRecord(b->join[i], c->stream));
                DFTG_CUDA(cudaStreamWaitEvent(s0, b->join[i], 0));
            }
        }
        return DFTG_OK;
    };
    auto mark_built = [&]() {
        for (dftg_ctx *c : b->ctx) {
            c->rho_scaled = true;
            if (persist) c->rw_ready = true;
            c->have_density = true;
            c->have_hartree = true;
            c->have_build = true;
            c->fwd_mask = c->prec_mask;
        }
        b->last = s0;
    };
    if (!b->exec) {
        if (!b->warm) {
            b->warm = true;
            b->key = key;
            DFTG_TRY(order_before());
            const int rc = enqueue();
            if (rc != DFTG_OK) return rc;
            mark_built();
            return order_after();
        }
        cudaGraph_t g = nullptr;
        DFTG_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue();
        const cudaError_t e = cudaStreamEndCapture(s0, &g);
        if (rc != DFTG_OK) {
            if (g) cudaGraphDestroy(g);
            return rc;
        }
        if (e != cudaSuccess) return cuda_fail(e, "cudaStreamEndCapture", __FILE__, __LINE__);
        const cudaError_t ei = cudaGraphInstantiate(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority);
        cudaGraphDestroy(g);
        if (ei != cudaSuccess) {
            b->exec = nullptr;
            return cuda_fail(ei, "cudaGraphInstantiate", __FILE__, __LINE__);
        }
    }
    DFTG_TRY(order_before());
    DFTG_CUDA(cudaGraphLaunch(b->exec, s0));
    mark_built();
    return order_after();
}

extern "C" int dftg_batch_set_mode(dftg_batch *b, int mode)
{
    if (!b) { set_error("null batch"); return DFTG_ERR_ARG; }
    if (mode != DFTG_BATCH_PERSISTENT && mode != DFTG_BATCH_GRAPH) { set_error("unknown batch mode %d", mode); return DFTG_ERR_ARG; }
    b->mode = mode;
    return DFTG_OK;
}

extern "C" int dftg_batch_get_mode(const dftg_batch *b, int *persistent_active)
{
    if (!b) { set_error("null batch"); return DFTG_ERR_ARG; }
    if (persistent_active) *persistent_active = b->plan != nullptr && b->mode == DFTG_BATCH_PERSISTENT ? 1 : 0;
    return b->mode;
}

// A CTA whose wait gave up stops, leaving the last-block counters of the
// reductions it skipped part-way: zero them all (the stream is synchronised)
static int reset_counters(dftg_batch *b)
{
    for (dftg_ctx *c : b->ctx) DFTG_CUDA(cudaMemset(c->d_counters, 0, sizeof(int) * dftg::kNumCounters));
    return DFTG_OK;
}

extern "C" int dftg_batch_status(dftg_batch *b)
{
    if (!b) { set_error("null batch"); return DFTG_ERR_ARG; }
    DFTG_CUDA(cudaSetDevice(b->ctx[0]->device));
    int code = 0;
    if (b->plan && b->last) DFTG_TRY(dftg::batch_plan_take_error(b->plan, b->last, &code));
    int rc = DFTG_OK;
    for (dftg_ctx *c : b->ctx) {
        const int r = sync_scalars(c);      // also reads and clears the context's bounded-wait flag
        if (r != DFTG_OK && rc == DFTG_OK) rc = r;
    }
    if (code) {
        DFTG_TRY(reset_counters(b));
        set_error("a bounded wait of the batch's persistent launches expired (code %d); results of this batch are invalid",
                  code);
        return DFTG_ERR_TIMEOUT;
    }
    return rc;
}

extern "C" int dftg_batch_selftest_wait(dftg_batch *b, double limit_ms)
{
    if (!b) { set_error("null batch"); return DFTG_ERR_ARG; }
    if (!(limit_ms > 0.0 && limit_ms <= 2000.0)) { set_error("limit_ms %g out of (0, 2000]", limit_ms); return DFTG_ERR_ARG; }
    if (!b->plan || !b->last) { set_error("self-test before a persistent batch build"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(b->ctx[0]->device));
    DFTG_TRY(dftg::batch_plan_enqueue(b->plan, b->last, 0, (unsigned long long)(limit_ms * 1e6), true));
    int code = 0;
    DFTG_TRY(dftg::batch_plan_take_error(b->plan, b->last, &code));
    for (dftg_ctx *c : b->ctx) c->have_build = c->have_hartree = false;   // the self-test left partial results
    if (code) {
        DFTG_TRY(reset_counters(b));
        set_error("a bounded wait of the batch's persistent launches expired (code %d)", code);
        return DFTG_ERR_TIMEOUT;
    }
    return DFTG_OK;
}

// Autotuner of a batch: the contexts' CTA counts scaled together by 1, 1/2,
// 1/4 and 1/8 (and 1/16, 1/32 in the persistent form: fewer, longer work items
// per molecule; in the graph form the branches run concurrently, so smaller
// grids per build can raise the throughput); every candidate is timed on the
// contexts' own density matrices and the fastest scale is kept.
extern "C" int dftg_batch_autotune(dftg_batch *b, int reps, double *best_ms)
{
    if (!b) { set_error("null batch"); return DFTG_ERR_ARG; }
    if (reps < 1) { set_error("reps < 1"); return DFTG_ERR_ARG; }
    const int n = (int)b->ctx.size();
    for (dftg_ctx *c : b->ctx)
        if (!c->have_build) { set_error("batch autotune before a complete build of every context"); return DFTG_ERR_STATE; }
    DFTG_CUDA(cudaSetDevice(b->ctx[0]->device));
    std::vector<const double *> P(n);
    std::vector<int> tc0(n), ct0(n);
    for (int i = 0; i < n; ++i) {
        P[i] = b->ctx[i]->d_P;
        tc0[i] = b->ctx[i]->tc_grid;
        ct0[i] = b->ctx[i]->ct_grid;
    }
    cudaStream_t s0 = b->ctx[0]->stream;
    auto run = [&](int div, double *ms) -> int {
        for (int i = 0; i < n; ++i) {
            dftg_ctx *c = b->ctx[i];
            if (c->tc_ready) c->tc_grid = std::max(1, tc0[i] / div);
            if (c->ct_ready) c->ct_grid = std::max(1, ct0[i] / div);
        }
        for (int w = 0; w < 2; ++w)   // eager, then capture
            DFTG_TRY(dftg_batch_fock_build_device(b, P.data(), nullptr, nullptr, nullptr, nullptr));
        cudaEvent_t e0, e1;
        DFTG_CUDA(cudaEventCreate(&e0));
        DFTG_CUDA(cudaEventCreate(&e1));
        int rc = cudaEventRecord(e0, s0) == cudaSuccess ? DFTG_OK : DFTG_ERR_CUDA;
        for (int r = 0; r < reps && rc == DFTG_OK; ++r)
            rc = dftg_batch_fock_build_device(b, P.data(), nullptr, nullptr, nullptr, nullptr);
        float t = 0.f;
        if (rc == DFTG_OK && cudaEventRecord(e1, s0) != cudaSuccess) rc = DFTG_ERR_CUDA;
        if (rc == DFTG_OK && cudaEventSynchronize(e1) != cudaSuccess) rc = DFTG_ERR_CUDA;
        if (rc == DFTG_OK && cudaEventElapsedTime(&t, e0, e1) != cudaSuccess) rc = DFTG_ERR_CUDA;
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        if (rc != DFTG_OK) { set_error("batch autotune timing failed"); return rc; }
        for (dftg_ctx *c : b->ctx) DFTG_TRY(sync_scalars(c));
        *ms = (double)t / reps;
        return DFTG_OK;
    };
    double best = 0.0;
    int best_div = 1;
    DFTG_TRY(run(1, &best));
    // the persistent form also tries fewer, longer work items per molecule
    const int ndiv = b->mode == DFTG_BATCH_PERSISTENT ? 5 : 3;
    const int divs[5] = {2, 4, 8, 16, 32};
    for (int k = 0; k < ndiv; ++k) {
        double t = 0.0;
        DFTG_TRY(run(divs[k], &t));
        if (t < best) { best = t; best_div = divs[k]; }
    }
    double t = 0.0;
    DFTG_TRY(run(best_div, &t));   // leave the chosen shapes and their outputs
    if (best_ms) *best_ms = best;
    return DFTG_OK;
}
