/*
 * dftg.h -- C ABI of the GB300-native grid Fock build (DFTCXX drop-in).
 *
 * Replaces the grid part of DFTCXX's MolecularGrid / AtomicGrid / DFT call
 * surface (ifilot/dftcxx, src/moleculargrid.h:84-167, src/atomicgrid.h:75-241,
 * src/dft.cpp:394-447).  Plain C types only: counts, host pointers and sizes.
 *
 * Conventions (identical to the reference):
 *   - lengths in bohr, energies in Hartree;
 *   - P is the closed-shell *half* density matrix: rho = 2 phi^T P phi
 *     (gridpoint.cpp:82-84);
 *   - J is returned such that F = H + 2 J + XC (dft.cpp:334); the 1/2 of
 *     atomicgrid.cpp:485 is inside J;
 *   - nbf x nbf matrices are column-major (Eigen's default); the matrices are
 *     symmetric, so row-major callers may pass them unchanged;
 *   - per-point arrays are ordered atom by atom, radial shell by shell
 *     (largest radius first), Lebedev point by point (atomicgrid.cpp:48-81).
 *
 * Errors: every call returns DFTG_OK (0) or a DFTG_ERR_* code; nothing throws
 * across the ABI.  dftg_last_error() gives a message for the calling thread.
 * Threading: one context per CUDA stream; calls on one context must be
 * serialised by the caller.  Different contexts may be used concurrently.
 * Ownership: the context owns all device memory; the caller owns every host
 * array it passes; no pointer is retained after a call returns.
 */
#ifndef DFTG_H
#define DFTG_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define DFTG_OK 0
#define DFTG_ERR_ARG 1        /* invalid argument or size */
#define DFTG_ERR_CUDA 2       /* CUDA runtime error (message has details) */
#define DFTG_ERR_NONFINITE 3  /* non-finite or asymmetric input matrix */
#define DFTG_ERR_STATE 4      /* call order violated (e.g. XC before density) */
#define DFTG_ERR_NOMEM 5      /* device allocation failed */
#define DFTG_ERR_TIMEOUT 6    /* a bounded device wait gave up */

/* arithmetic of the per-iteration build */
#define DFTG_PREC_FP64 0      /* every step in FP64 on the CUDA cores */
#define DFTG_PREC_MIXED 1     /* contractions split-precision, FP64 reductions */

/* Lebedev orders: 0..10 are the reference's enum (settings.h:64-78:
 * 6,14,26,38,50,74,86,110,146,170,194 points); 11 is the 302-point rule, an
 * extension generated from the published Lebedev-Laikov data. */
#define DFTG_LEBEDEV_302 11

typedef struct dftg_ctx dftg_ctx;

/* Atoms: replaces Molecule's atom list (molecule.h:41-81, molecule.cpp:97-101). */
typedef struct {
    int natoms;
    const int *Z;          /* [natoms] nuclear charges (1..18) */
    const double *xyz;     /* [natoms][3] bohr */
} dftg_molecule;

/* Contracted Cartesian Gaussians: replaces Molecule's CGF list (cgf.h:152-287,
 * molecule.cpp:135-238).  Function i sits on atom bf_atom[i] with powers
 * bf_lmn[3i..3i+2] and bf_nprim[i] primitives taken in order from prim_alpha /
 * prim_coef.  Primitive normalisation follows cgf.cpp:102-114. */
typedef struct {
    int nbf;
    const int *bf_atom;       /* [nbf] */
    const int *bf_lmn;        /* [nbf][3] */
    const int *bf_nprim;      /* [nbf] */
    const double *prim_alpha; /* [sum(bf_nprim)] */
    const double *prim_coef;  /* [sum(bf_nprim)] */
} dftg_basis;

/* MolecularGrid::set_grid_parameters (moleculargrid.cpp:175-179). */
typedef struct {
    int radial_points;     /* Gauss-Chebyshev radial points per atom, >= 8 */
    int lebedev_order;     /* 0..11, see above */
    int lmax;              /* spherical-harmonic cut-off of the Hartree solve, 0..16 */
    int device;            /* CUDA device ordinal */
} dftg_grid_params;

/* Build molecule, basis and grid: MolecularGrid(mol) + create_grid()
 * (moleculargrid.cpp:31-34, 193-261).  Computes grid points, Becke weights and
 * the basis amplitudes on the device. */
int dftg_create(const dftg_molecule *mol, const dftg_basis *basis,
                const dftg_grid_params *grid, dftg_ctx **out);
int dftg_destroy(dftg_ctx *ctx);
const char *dftg_last_error(void);

/* Sizes. */
int dftg_grid_size(const dftg_ctx *ctx, size_t *npts);   /* grid_size, moleculargrid.h:76 */
int dftg_nbf(const dftg_ctx *ctx, int *nbf);             /* Molecule::get_nr_bfs */

/* Precision of the per-iteration build (default DFTG_PREC_FP64). */
int dftg_set_precision(dftg_ctx *ctx, int precision);
/* Finer control for error budgets (no counterpart in the reference): each set
 * bit runs one step of the build in the mixed form, the others in FP64.
 * DFTG_PREC_MIXED is all bits; 0 is DFTG_PREC_FP64. */
#define DFTG_MIX_DENSITY 1u     /* rho = 2 phi^T P phi */
#define DFTG_MIX_LDA 2u         /* Slater + VWN point kernel */
#define DFTG_MIX_MULTIPOLE 4u   /* rho_lm projection and own-cell potential */
#define DFTG_MIX_CROSS 8u       /* cross-atom Hartree potential */
#define DFTG_MIX_CONTRACT 16u   /* XC and J contractions */
int dftg_set_precision_mask(dftg_ctx *ctx, unsigned mask);
/* Run on a caller-owned cudaStream_t (one the caller created).  NULL does NOT
 * mean the legacy default stream here: it restores the context's own stream,
 * which is non-blocking, so it is not ordered with work on the legacy default
 * stream.  The builds are replayed as CUDA graphs captured on the stream, and
 * the legacy and per-thread default streams cannot be captured, so
 * cudaStreamLegacy and cudaStreamPerThread are rejected (DFTG_ERR_ARG).  A
 * caller whose work is on a default stream synchronises it first, or moves it
 * to a stream it created and passes that one. */
int dftg_set_stream(dftg_ctx *ctx, void *cuda_stream);

/* MolecularGrid::set_density(P) (moleculargrid.cpp:48-53): rho = 2 phi^T P phi
 * on every point.  P: nbf x nbf host array. */
int dftg_set_density(dftg_ctx *ctx, const double *P);
/* MolecularGrid::correct_densities (moleculargrid.cpp:132-146): scales rho by
 * sum(Z) / integral(w rho); the factor is written to *scale (may be NULL). */
int dftg_correct_densities(dftg_ctx *ctx, double *scale);
/* MolecularGrid::calculate_density (moleculargrid.cpp:157-166). */
int dftg_calculate_density(dftg_ctx *ctx, double *nelec);
/* MolecularGrid::calculate_hartree_potential (moleculargrid.cpp:336-389):
 * Becke-Poisson Hartree potential on every point and J (nbf x nbf). */
int dftg_calculate_hartree_potential(dftg_ctx *ctx, double *J);
/* DFT::calculate_exchange_correlation_matrix (dft.cpp:394-433): Slater +
 * VWN point kernel, XC (nbf x nbf) and E_xc. */
int dftg_calculate_xc(dftg_ctx *ctx, double *XC, double *exc);

/* One whole grid Fock build at fixed P (dft.cpp:361-365, 377-433): the four
 * calls above in one, with host buffers.  Any output pointer may be NULL. */
int dftg_fock_build(dftg_ctx *ctx, const double *P, double *J, double *XC,
                    double *exc, double *nelec);
/* The same with DEVICE pointers on the context's stream and no host
 * synchronisation (P: nbf*nbf doubles; J, XC: nbf*nbf; scalars: a 3-double
 * device array receiving E_xc, the integrated density and E_J).  For callers
 * whose P is already in HBM. */
int dftg_fock_build_device(dftg_ctx *ctx, const double *P_dev, double *J_dev,
                           double *XC_dev, double *scalars_dev);

/* Energies of the last build: E_xc, E_J and the integrated density.  E_J is
 * the Hartree term of DFT::calculate_energy, 2 tr(P J) (dft.cpp:443), which
 * equals sum_p (w_p V_p / 2) rho_p over the grid with rho = 2 phi^T P phi
 * before correction; it is summed on the grid in FP64 in both precisions, so
 * the energy does not inherit the split-precision rounding of the J matrix. */
int dftg_get_energies(dftg_ctx *ctx, double *exc, double *ej, double *nelec);

/* Diagnostic variant of dftg_fock_build_device (no counterpart in the
 * reference, which only prints wall-clock totals, dft.cpp:98-119): runs one
 * build with CUDA events between the kernel phases and returns up to cap
 * per-phase durations in milliseconds with their names (static strings).  On a
 * point-set context it profiles the step of dftg_xc_build_device instead. */
int dftg_fock_build_profile(dftg_ctx *ctx, const double *P_dev, double *phase_ms,
                            const char **names, int cap, int *nphase);

/* Point-set context (no counterpart in the reference): the amplitude, density,
 * LDA and XC steps on explicit points with explicit weights, for contraction
 * workloads without a molecular grid.  centres->xyz gives the function centres
 * (bf_atom indexes them; centres->Z is ignored).  Such a context supports
 * dftg_set_density (rho = 2 phi^T P phi, no density correction),
 * dftg_calculate_density, dftg_calculate_xc, dftg_xc_build*, the getters and
 * the launch-shape calls; calls that need nuclei or the Hartree step return
 * DFTG_ERR_STATE. */
typedef struct {
    size_t npts;
    const double *xyz;     /* [npts][3] bohr */
    const double *w;       /* [npts] quadrature weights */
} dftg_points;
int dftg_create_points(const dftg_points *pts, const dftg_molecule *centres, const dftg_basis *basis, int device,
                       dftg_ctx **ctx);

/* rho, the LDA point kernel and XC = phi^T diag(w v_xc) phi in one call, on any
 * context, without the density correction (DFT::calculate_exchange_correlation_matrix,
 * dft.cpp:394-433, for a fixed rho).  XC may be NULL; exc and nelec (the
 * integral of w rho) may be NULL.  The device form writes scalars_dev[0] = E_xc,
 * [1] = the integral, and does not synchronise. */
int dftg_xc_build(dftg_ctx *ctx, const double *P, double *XC, double *exc, double *nelec);
int dftg_xc_build_device(dftg_ctx *ctx, const double *P_dev, double *XC_dev, double *scalars_dev);

/* Atom-cell shards (no counterpart in the reference, which keeps one
 * AtomicGrid per atom in one process: moleculargrid.cpp:193-261, 336-389).
 * For several GPUs, or several processes, the build is split by fuzzy cell:
 * every rank creates a context over the cells of atoms [first_cell,
 * first_cell + ncells) of the same molecule (the grid points of those cells;
 * Becke weights, basis functions and the cross-atom potential still see every
 * atom) and runs the three calls below, with three exchanges between them:
 *   1. dftg_shard_density: rho on the shard's points (P: host nbf x nbf);
 *      *sum_wrho = the shard's integral of w rho.  Exchange: all-reduce (sum)
 *      of sum_wrho over the ranks = the molecule's integral.
 *   2. dftg_shard_multipoles(total): the correction factor sum(Z) / total
 *      (moleculargrid.cpp:132-146), the LDA point kernel, and rho_lm, the
 *      Poisson solve, the own-cell potential and the spline data of the
 *      shard's cells, written to blob [ncells][per-cell doubles] (see
 *      dftg_shard_blob_size).  Exchange: all-gather of the blobs in cell order
 *      = [natoms][per-cell doubles].
 *   3. dftg_shard_finish(blob_all): the cross-atom potential on the shard's
 *      points from every cell's splines, and the shard's parts of J, XC (host
 *      nbf x nbf, either may be NULL) and scalars = {E_xc, integral of the
 *      corrected rho, E_J}.  Exchange: all-reduce (sum) of J, XC and scalars =
 *      the whole build's.
 * The blobs are opaque doubles (FP64 and split FP32 spline tables) that must
 * travel bit for bit.  The whole-molecule build calls (dftg_fock_build*,
 * dftg_correct_densities, dftg_calculate_hartree_potential, backward, SCF,
 * batches) return DFTG_ERR_STATE on a shard context; dftg_set_density,
 * dftg_calculate_density and the getters act on the shard's points. */
int dftg_create_cells(const dftg_molecule *mol, const dftg_basis *basis, const dftg_grid_params *grid,
                      int first_cell, int ncells, dftg_ctx **out);
int dftg_shard_blob_size(const dftg_ctx *ctx, size_t *doubles_per_cell, int *first_cell, int *ncells);
int dftg_shard_density(dftg_ctx *ctx, const double *P, double *sum_wrho);
int dftg_shard_multipoles(dftg_ctx *ctx, double total_wrho, double *blob, size_t cap);
int dftg_shard_finish(dftg_ctx *ctx, const double *blob_all, size_t cap, double *J, double *XC, double *scalars);

/* Getters (copies): MolecularGrid::get_weights / get_densities /
 * get_amplitudes (moleculargrid.cpp:61-127).  cap is the element capacity of
 * out.  Amplitudes are nbf x npts column-major (the reference's layout). */
int dftg_get_weights(const dftg_ctx *ctx, double *out, size_t cap);
int dftg_get_becke_weights(const dftg_ctx *ctx, double *out, size_t cap);
int dftg_get_densities(const dftg_ctx *ctx, double *out, size_t cap);
int dftg_get_amplitudes(const dftg_ctx *ctx, double *out, size_t cap);
int dftg_get_positions(const dftg_ctx *ctx, double *out, size_t cap);   /* [npts][3] */
int dftg_get_potential(const dftg_ctx *ctx, double *out, size_t cap);   /* Hartree V */

/* One-electron matrices S, T, V (sum over nuclei) and E_nuc, computed on the
 * device in FP64 (DFT::construct_matrices dft.cpp:184-199, integrals.cpp:43-387,
 * gamma.cpp:41-229).  Any pointer may be NULL. */
int dftg_one_electron(dftg_ctx *ctx, double *S, double *T, double *V);
int dftg_nuclear_repulsion(const dftg_ctx *ctx, double *enuc);

/* The reference's analytic Hartree path (Settings::TWO_ELECTRON_INTEGRALS):
 * J_ij = sum_kl P_kl (ij|kl) (DFT::calculate_hartree_potential_te_int,
 * dft.cpp:452-477) from two-electron integrals over the context's basis
 * (DFT::calculate_two_electron_integrals dft.cpp:254-288, Integrator::repulsion
 * integrals.cpp:185-466), computed on the device in FP64 (McMurchie-Davidson)
 * without storing the integrals.  An independent check of the grid J of
 * dftg_calculate_hartree_potential; s, p and d functions.  P, J: host nbf x nbf. */
int dftg_eri_coulomb(dftg_ctx *ctx, const double *P, double *J);
/* Every unique (ij|kl) at the reference's teindex position (integrals.cpp:470-486):
 * pair ij = i(i+1)/2 + j (i >= j), index ij(ij+1)/2 + kl (ij >= kl);
 * T(T+1)/2 values with T = nbf(nbf+1)/2.  cap: capacity of out in doubles. */
int dftg_eri_list(dftg_ctx *ctx, double *out, size_t cap);

/* Backward pass of the grid energy (no counterpart in the reference; the
 * forward is the last complete Fock build on the context: dftg_fock_build,
 * dftg_fock_build_device or a batch).  With E = seed_exc * E_xc + seed_ej * E_J,
 * E_J = 2 tr(P J), computed by that build, writes
 *   dEdP [nbf x nbf]  dE/dP_{mu nu}, every element of P taken as independent
 *                     (symmetric; E changes by sum dEdP .* dP for a change dP),
 *   dEdR [natoms][3]  dE/dR at fixed P: basis functions and grid points move
 *                     with their atoms (amplitude gradients, Becke-weight
 *                     derivatives, cross-atom potential geometry).  The grid
 *                     part of the nuclear forces is -dEdR.
 * Either output may be NULL.  The forward state (density, potential, weights)
 * is read, not changed, except that the FP64 multipole work arrays are
 * recomputed.  Errors: DFTG_ERR_STATE without a preceding complete build;
 * DFTG_ERR_ARG for lmax > 13 or an amplitude block too large for shared memory. */
int dftg_backward(dftg_ctx *ctx, double seed_exc, double seed_ej, double *dEdP, double *dEdR);
/* The same on device buffers, ordered on the context's stream, no synchronisation. */
int dftg_backward_device(dftg_ctx *ctx, double seed_exc, double seed_ej, double *dEdP_dev, double *dEdR_dev);
/* Diagnostic variant of dftg_backward (both outputs, kept on the device):
 * per-phase durations in milliseconds with their names, as
 * dftg_fock_build_profile. */
int dftg_backward_profile(dftg_ctx *ctx, double seed_exc, double seed_ej, double *phase_ms, const char **names,
                          int cap, int *nphase);

/* Batched builds (no counterpart in the reference; its driver builds one
 * molecule at a time, dft.cpp:84-142): many contexts -- molecules or
 * geometries of any size -- built together.  Two forms:
 *   DFTG_BATCH_PERSISTENT (default): every step of the mixed build runs as ONE
 *     persistent launch over all contexts (eight launches per batch, the LDA
 *     point kernel on a second branch beside the Hartree launches); each CTA
 *     takes (context, block) work items from a device queue and runs each as
 *     that block of the context's own launch, so every context's results are
 *     bit-identical to its single build.  The point-kernel launch can also
 *     take per-atom sum items, whose context's point blocks then wait,
 *     bounded (2 s), for the correction factor; every context a batch accepts
 *     gets its factor from the density launch instead, so no block waits in a
 *     build.  A wait that gives up is reported by dftg_batch_status.  Needs
 *     every context in mixed precision with the
 *     tensor-core density and contraction (nbf <= 80) and <= 256 radial points;
 *     otherwise the batch falls back to the graph of branches.
 *   DFTG_BATCH_GRAPH: each context's kernel sequence on its own stream branch
 *     of one CUDA graph (any precision, any size).
 * Either way the launches are captured into a CUDA graph and replayed: the
 * first call with a new set of buffers runs eagerly and the next one
 * captures.  The contexts must be distinct and stay alive while the batch
 * exists. */
#define DFTG_BATCH_PERSISTENT 0
#define DFTG_BATCH_GRAPH 1
typedef struct dftg_batch dftg_batch;
int dftg_batch_create(dftg_ctx *const *ctxs, int n, dftg_batch **out);
int dftg_batch_destroy(dftg_batch *b);
/* Select the form (takes effect at the next build).  dftg_batch_get_mode
 * returns the selected form and sets *persistent_active (may be NULL) to 1 when
 * the last build ran as persistent launches. */
int dftg_batch_set_mode(dftg_batch *b, int mode);
int dftg_batch_get_mode(const dftg_batch *b, int *persistent_active);
/* Synchronise the batch's last launch and report its bounded waits:
 * DFTG_ERR_TIMEOUT when one gave up (the flags are cleared), else DFTG_OK. */
int dftg_batch_status(dftg_batch *b);
/* Self-test of the persistent batch's bounded wait: runs the atom-sum + point
 * launch with one point item of the first context, which waits on a flag that
 * nothing sets, limit limit_ms (0 < limit_ms <= 2000); returns DFTG_ERR_TIMEOUT.  The
 * contexts' results are then incomplete until their next build (DFTG_ERR_STATE
 * for calls that need one).  Needs a preceding persistent build. */
int dftg_batch_selftest_wait(dftg_batch *b, double limit_ms);
/* dftg_fock_build_device for every context i with P_devs[i], J_devs[i],
 * XC_devs[i], scalars_devs[i] (arrays of n device pointers; J, XC and scalars
 * entries may be NULL).  stream: a cudaStream_t the batch is ordered on: its
 * branches start after the work queued there before the call, and the stream
 * waits for all of them, so events recorded on it bracket the whole batch.
 * NULL does NOT mean the legacy default stream: it selects the first context's
 * own (non-blocking) stream, which is not ordered after legacy-stream work (a
 * fill of the outputs, a copy of P); the default streams themselves cannot be
 * captured and are rejected (DFTG_ERR_ARG), as in dftg_set_stream.  The call
 * returns without synchronising. */
int dftg_batch_fock_build_device(dftg_batch *b, const double *const *P_devs, double *const *J_devs,
                                 double *const *XC_devs, double *const *scalars_devs, void *stream);
/* Batch autotuner: scales every context's CTA counts by 1, 1/2, 1/4 and 1/8
 * together, and 1/16 and 1/32 in the persistent form (fewer, longer work items
 * per molecule there; concurrent branches in the graph form), times reps replays of the batch on the
 * contexts' own last P and keeps the fastest scale; needs a complete build of
 * every context.  best_ms (per batch replay) may be NULL. */
int dftg_batch_autotune(dftg_batch *b, int reps, double *best_ms);

/* Launch-shape autotuner (no counterpart in the reference).  Shape =
 * {CTAs of the tensor-core density kernel, CTAs of the tensor-core XC / J
 * contraction, pipeline stages of the contraction (even)}; 0 where the context
 * has no such kernel.  dftg_autotune times reps graph-replayed builds of the last
 * built P for candidate shapes (coordinate descent, each knob from the current
 * best) and keeps the fastest; it needs a preceding complete build and leaves
 * the outputs of a build with the chosen shape.  best_ms may be NULL. */
int dftg_get_launch_shape(const dftg_ctx *ctx, int *shape, int cap);
int dftg_set_launch_shape(dftg_ctx *ctx, const int *shape, int n);
int dftg_autotune(dftg_ctx *ctx, int reps, double *best_ms);

/* Self-test of the bounded-wait error path (no counterpart in the reference).
 * Every spin-wait of the tensor-core kernels is bounded; on expiry the kernel
 * records an error code and exits, and the host call returns DFTG_ERR_TIMEOUT.
 * This launches one warp that waits on an mbarrier that nothing arrives at,
 * with a limit of limit_ms (0 < limit_ms <= 2000), and returns what a build
 * would: DFTG_ERR_TIMEOUT.  The context stays usable. */
int dftg_selftest_wait(dftg_ctx *ctx, double limit_ms);

/* XC and J contraction that allocates nothing.  No counterpart in the
 * reference: it exists for callers that may not call cudaMalloc / cudaFree
 * while serving (their framework owns all device memory, or they run under a
 * fixed device-memory budget).  Computes, in FP64,
 *   XC = phi^T diag(cxc) phi,   J = phi^T diag(cj) phi
 * from caller-owned device buffers on the current device: phi is nbf rows of
 * npts amplitudes, row stride ld (>= npts) doubles; cxc, cj hold npts point
 * coefficients; XC and J (nbf x nbf, either may be NULL) are written.  Its
 * scratch is a static device array of DFTG_NOALLOC_SCRATCH_BYTES that every GPU
 * loading the library holds until exit; nbf above DFTG_NOALLOC_MAX_NBF is
 * rejected with DFTG_ERR_ARG.  Every call looks up that array's address on the
 * current device (no allocation); the first call on a device also loads the
 * library's device code there, so make it before any stream capture.  Calls
 * that overlap on the GPU race on the shared array.  stream: a cudaStream_t,
 * NULL for the legacy default stream (as in the CUDA runtime); the call
 * returns without synchronising. */
#define DFTG_NOALLOC_SCRATCH_BYTES (16u * 1024u * 1024u)
#define DFTG_NOALLOC_MAX_NBF 1024
int dftg_contract_noalloc(const double *phi, size_t ld, size_t npts, int nbf,
                          const double *cxc, const double *cj, double *XC,
                          double *J, void *stream);

/* Device SCF driver: the reference's DFT constructor and DFT::scf
 * (dft.cpp:57-61, 84-142, 160-227, 300-366, 441-447) with every step on the
 * GPU.  Per iteration: F = H + 2J + XC, F' = X^T F X, eigen-decomposition of F'
 * (FP32 Jacobi rotations in one CTA, then FP64 iterative refinement that
 * separates the occupied and virtual subspaces to FP64 accuracy),
 * P_new = C_occ C_occ^T with C = X C', P <- (1 - alpha) P_new + alpha P, the
 * grid Fock build of this context (its precision), and
 * E = 2 tr(P H) + E_J + E_nuc + E_xc (E_J = 2 tr(P J) in FP64 builds, the FP64
 * grid sum in mixed builds).  X = U diag(lambda^-1/2) from the eigenpairs of S,
 * polished in FP64 until X^T S X = I.  dftg_scf_run runs the whole loop as one
 * CUDA graph launch (a conditional while node whose body ends with the
 * convergence test), so the host waits once per SCF, not once per iteration. */
typedef struct dftg_scf_params {
    int nelec;         /* electrons (even); 0: sum of Z (neutral molecule) */
    double alpha;      /* weight of the old P in the damping (reference: 0.5) */
    double tol;        /* stop when |E_n - E_(n-1)| <= tol (reference: 1e-4) */
    int min_iter;      /* at least this many iterations (reference: 3) */
    int max_iter;      /* at most this many, <= DFTG_SCF_MAX_ITER (reference: 100) */
    int refine_steps;  /* FP64 refinement steps per eigen-solve; 0: default 4 */
} dftg_scf_params;
#define DFTG_SCF_MAX_NBF 160
#define DFTG_SCF_MAX_ITER 1000
/* Set-up (the reference's DFT constructor + construct_matrices): S, T, V, H,
 * E_nuc, X, the first density from H, its Hartree J and the energy E_0 with
 * E_xc = 0.  nbf <= DFTG_SCF_MAX_NBF.  Errors: DFTG_ERR_ARG for bad parameters,
 * DFTG_ERR_STATE for a point-set context or an S that is not positive definite. */
int dftg_scf_init(dftg_ctx *ctx, const dftg_scf_params *params);
/* Iterate to convergence (or max_iter).  energy: final E; iterations: count.
 * Calling it again continues from the current P (as a second DFT::scf would). */
int dftg_scf_run(dftg_ctx *ctx, double *energy, int *iterations);
/* One iteration, synchronised (for host-driven loops).  energy: its E;
 * converged: 1 when the reference's loop would stop after this iteration. */
int dftg_scf_step(dftg_ctx *ctx, double *energy, int *converged);
/* Results.  DFTG_SCF_P, _J, _XC, _H, _X: nbf x nbf; DFTG_SCF_EPS: the nbf
 * orbital energies ascending; DFTG_SCF_COCC: the occupied coefficients
 * [nocc columns of nbf]; DFTG_SCF_HISTORY: DFTG_SCF_HIST_W values per
 * iteration {E, 2tr(PH), E_J, E_xc, N, |dE|} of the last run; DFTG_SCF_DIAG:
 * {max |S'_ij| between occupied and virtual vectors, max |I - C'^T C'|, Jacobi
 * sweeps, mode (1: conditional-graph loop, 2: host-stepped graphs)} of the last
 * eigen-solve; DFTG_SCF_STATE: {E (E_0 after dftg_scf_init), iterations of the
 * current run, last |dE|, 1 if the loop would continue}.  cap: capacity of out
 * in doubles; n: values written (may be NULL). */
#define DFTG_SCF_P 0
#define DFTG_SCF_J 1
#define DFTG_SCF_XC 2
#define DFTG_SCF_H 3
#define DFTG_SCF_X 4
#define DFTG_SCF_EPS 5
#define DFTG_SCF_COCC 6
#define DFTG_SCF_HISTORY 7
#define DFTG_SCF_DIAG 8
#define DFTG_SCF_STATE 9
#define DFTG_SCF_HIST_W 6
int dftg_scf_get(dftg_ctx *ctx, int what, double *out, size_t cap, size_t *n);

#ifdef __cplusplus
}
#endif

#endif /* DFTG_H */
