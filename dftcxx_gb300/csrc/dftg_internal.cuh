// dftg_internal.cuh -- context layout and kernel launchers of the grid Fock build.
//
// Data layout in HBM (npad = grid size rounded up to 128; padded points carry
// zero weight and zero amplitudes so every kernel can work on whole tiles):
//   points      X, Y, Zc, W, WB, rho, V     [npad] FP64 (structure of arrays)
//   amplitudes  phi   [nbf][npad] FP64      (point-contiguous per function)
//               phi32 [nbf][npad] FP32      (mixed-precision copy)
//   point coefficients  cxc = w*v_xc, cj = w*V/2   [npad] FP64 and FP32
//   Hartree     Y [nlm][nang], rholm/U [natoms][nlm][nrad], LU factors per l,
//               spline coefficients [natoms][nlm][nrad][4] (last interval = clamp)
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

void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what, const char *file, int line);

#define DFTG_CUDA(call)                                                        \
    do {                                                                       \
        cudaError_t e_ = (call);                                               \
        if (e_ != cudaSuccess) return ::dftg::cuda_fail(e_, #call, __FILE__, __LINE__); \
    } while (0)

#define DFTG_LAUNCH_CHECK() DFTG_CUDA(cudaGetLastError())

}  // namespace dftg

struct dftg_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    int precision = DFTG_PREC_FP64;

    // molecule and basis (host copies)
    int natoms = 0, nbf = 0, nprim = 0;
    std::vector<int> Z;
    std::vector<double> xyz;
    std::vector<int> bf_atom, bf_lmn, bf_off;
    std::vector<double> alpha, coef, norm;

    // grid
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
    double *d_cxc = nullptr, *d_cj = nullptr;
    float *d_cxc32 = nullptr, *d_cj32 = nullptr;
    double *d_phi = nullptr;
    float *d_phi32 = nullptr;

    // device: matrices
    double *d_P = nullptr;
    float *d_P32 = nullptr;
    double *d_J = nullptr, *d_XC = nullptr;
    double *d_part = nullptr;     // contraction partials [nchunk][2][nbf][nbf]
    size_t part_elems = 0;
    int nchunk = 0;               // point chunks of the contraction
    int ntiles = 0;               // output blocks on or above the diagonal
    void *d_tiles = nullptr;      // [ntiles] int2 block coordinates
    double *d_red = nullptr;      // reduction partials
    size_t red_elems = 0;
    double *d_scal = nullptr;     // scalars, see kScal* below
    double *h_scal = nullptr;     // pinned host mirror of d_scal

    // device: Hartree
    double *d_Y = nullptr;        // [nlm][nang] Y_lm of the Lebedev directions
    double *d_Yw = nullptr;       // [nlm][nang] w_leb * Y_lm
    double *d_pre = nullptr;      // [nlm] spherical-harmonic prefactors
    float *d_pre32 = nullptr;
    double *d_rec = nullptr;      // [nlm][2] associated-Legendre recursion coefficients
    float *d_rec32 = nullptr;
    double *d_rholm = nullptr;    // [natoms][nlm][nrad]
    double *d_U = nullptr;        // [natoms][nlm][nrad]
    double *d_LU = nullptr;       // [lmax+1][S][S] packed LU factors, S = nrad+2
    int *d_piv = nullptr;         // [lmax+1][S]
    double *d_sx = nullptr;       // [nrad] increasing spline abscissae
    double *d_spl = nullptr;      // [natoms][nrad-1][nlm][4]
    float *d_spl32 = nullptr;     // same in FP32

    // device: one-electron integrals output (allocated on first use)
    double *d_ints_work = nullptr;

    // call-order state
    bool have_density = false;
    bool have_hartree = false;

    // per-phase CUDA-event timing (dftg_fock_build_profile)
    static constexpr int kMaxMarks = 24;
    cudaEvent_t prof_ev[kMaxMarks] = {};
    const char *prof_name[kMaxMarks] = {};
    int prof_n = 0;
    bool prof_on = false;
};

namespace dftg {

// scalar slots in d_scal
enum {
    kScalSum = 0,      // sum_p w rho (before correction)
    kScalScale = 1,    // correction factor
    kScalExc = 2,      // E_xc
    kScalNelec = 3,    // integral of corrected rho
    kScalAtomQ = 8,    // [natoms] per-atom integral of rho (after correction)
};
inline size_t scal_elems(int natoms) { return 8 + (size_t)natoms; }

// records a named event after the preceding launch when profiling is on
int mark(dftg_ctx *c, const char *name);
#define DFTG_MARK(c, name) do { if ((c)->prof_on) { int rc_m_ = ::dftg::mark((c), (name)); if (rc_m_) return rc_m_; } } while (0)

// k_grid.cu
int launch_grid(dftg_ctx *c);
int launch_amplitudes(dftg_ctx *c);
// k_density.cu
int launch_density(dftg_ctx *c);
int launch_atom_sums(dftg_ctx *c, bool apply_scale);
int launch_xc_points(dftg_ctx *c);
int launch_convert_P(dftg_ctx *c);
// k_hartree.cu
int hartree_setup(dftg_ctx *c);
int launch_hartree(dftg_ctx *c);
// k_integrals.cu
int launch_one_electron(dftg_ctx *c, double *dS, double *dT, double *dV);
// k_contract.cu
int contract_setup(dftg_ctx *c);
size_t contract_part_elems(int nbf, size_t npad);
size_t reduction_elems(size_t npad, int natoms, int nrad, int nang);
int launch_contract(dftg_ctx *c, bool want_xc, bool want_j);

}  // namespace dftg
