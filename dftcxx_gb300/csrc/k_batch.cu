// k_batch.cu -- persistent launches of a batch of grid Fock builds (no
// counterpart in the reference, whose driver builds one molecule at a time:
// dft.cpp:84-142).
//
// Every step of the mixed build runs as ONE persistent launch over all of the
// batch's molecules.  A step's work items are the blocks of the molecules' own
// launches of that step (molecule-major); each CTA takes runs of items from a
// device counter and runs each item exactly as that block of the molecule's
// single launch (GroupQueue in dftg_internal.cuh), so every molecule's results
// are bit-identical to its own build.  Per batch: one memset of the queue
// counters, then nine launches --
//   P slices (with the copy of P into the context and the correction factor
//   from 2 tr(P S_grid)), density (tensor cores), LDA point kernel (with the
//   correction), multipole chain, cross-atom bins, potential gather + E_J,
//   coefficient bounds, XC / J contraction (tensor cores), partial reduction
//   (which also writes the caller's output buffers and scalars).  The point
//   kernel and the three Hartree launches are independent and run on two
//   branches (the Hartree ones on a stream of the greatest priority).
// The point-kernel launch also takes per-atom sum items for molecules without
// S_grid; their point blocks wait (bounded) for the molecule's factor.  Every
// context a batch accepts has S_grid, so no block waits but in the self-test of
// the bounded wait.
// The launch records of every molecule (arguments, block counts, shared memory)
// come from the same step functions the single build launches with, and are
// copied to the device once per set of buffers.
#include <algorithm>
#include <cstring>
#include <vector>
#include "dftg_internal.cuh"

namespace dftg {

enum {
    kStSliceP, kStDensity, kStSums, kStLda, kStMultipole, kStVcb, kStGather, kStCexp, kStContract, kStReduce,
    kNumSteps
};
// items a CTA takes per visit to the counter (the small point-block steps take
// several, so the counter is not the bottleneck)
static const int kTake[kNumSteps] = {4, 1, 4, 4, 1, 4, 2, 4, 1, 1};
constexpr int kCtlInts = 16;                 // queue counters, then the error flag at kCtlInts

struct BatchPlan {
    int nmol = 0, nsm = 0, device = 0, lmax = -1;
    void *d_mem = nullptr;
    int *d_heads = nullptr;                  // [kNumSteps] counters, then done[nmol]
    int *d_done = nullptr;
    int *d_err = nullptr;
    const int *d_self_prefix = nullptr;      // [nmol + 1] one point item, of molecule 0 (the wait self-test)
    size_t zero_bytes = 0;                   // counters and done flags, cleared before every batch
    GroupQueue q[kNumSteps];
    size_t smem[kNumSteps] = {};
    const void *args[kNumSteps] = {};
    // the Hartree steps' branch (greatest priority) beside the point-kernel launch
    cudaStream_t aux = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
};

bool batch_group_eligible(const dftg_ctx *c)
{
    return !c->points_only && c->cell0 == 0 && c->ncell == c->natoms && (c->prec_mask & kPrecAll) == kPrecAll &&
           c->tc_ready && c->ct_ready && c->nrad <= 256 && c->nlebpair > 0 && c->d_rw32 != nullptr;
}

void batch_plan_free(BatchPlan *bp)
{
    if (!bp) return;
    if (bp->d_mem) cudaFree(bp->d_mem);
    if (bp->aux) cudaStreamDestroy(bp->aux);
    if (bp->ev_fork) cudaEventDestroy(bp->ev_fork);
    if (bp->ev_join) cudaEventDestroy(bp->ev_join);
    delete bp;
}

static size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

int batch_plan_create(dftg_ctx *const *ctx, int n, const double *const *P, double *const *J, double *const *XC,
                      double *const *sc, BatchPlan **out)
{
    *out = nullptr;
    std::vector<StepLaunch<SlicePArgs>> s0(n);
    std::vector<StepLaunch<DensTcArgs>> s1(n);
    std::vector<StepLaunch<SumsArgs>> s2(n);
    std::vector<StepLaunch<LdaArgs>> s3(n);
    std::vector<StepLaunch<MpArgs>> s4(n);
    std::vector<StepLaunch<VcbArgs>> s5(n);
    std::vector<StepLaunch<GoArgs>> s6(n);
    std::vector<StepLaunch<CexpArgs>> s7(n);
    std::vector<StepLaunch<CtArgs>> s8(n);
    std::vector<StepLaunch<RedArgs>> s9(n);
    int lmax = ctx[0]->lmax;
    for (int i = 0; i < n; ++i) {
        // the launch records take the whole build's forms (cmax_route)
        struct WholeBuild {
            dftg_ctx *c;
            ~WholeBuild() { c->whole_build = false; }
        } whole{ctx[i]};
        ctx[i]->whole_build = true;
        const dftg_ctx *c = ctx[i];
        if (!batch_group_eligible(c)) { set_error("context %d cannot join a persistent batch", i); return DFTG_ERR_STATE; }
        if (c->lmax != lmax) lmax = -1;
        s0[i] = step_slice_P(c, P[i], P[i] != c->d_P ? c->d_P : nullptr, true);
        s1[i] = step_density_tc(c, true);
        s2[i] = step_atom_sums(c, kSumsFactor);
        const bool route = sgrid_route(c);
        // on the S_grid route the P-slicing step writes the factor and the density
        // epilogue corrects rho and writes the rho w_becke planes
        s3[i] = route ? step_lda(c, false, true, false) : step_lda(c, true, true, true);
        if (route) s2[i].blocks = 0;
        s4[i] = step_multipole(c, route ? rw_planes(c) : s3[i].args.rw32 != nullptr);
        s5[i] = step_vcross_bins(c);
        s6[i] = step_gather_own(c, true);
        s7[i] = step_cexp(c, c->d_cxc32, c->d_cj32);
        if (cmax_route(c)) s7[i].blocks = 0;   // the point kernel and the gather keep the chunk maxima
        s8[i] = step_contract_tc(c, c->d_cxc32, c->d_cj32);
        s9[i] = step_contract_reduce(c, true, true, c->d_XC, c->d_J);
        s9[i].args.XC2 = (XC && XC[i] && XC[i] != c->d_XC) ? XC[i] : nullptr;
        s9[i].args.J2 = (J && J[i] && J[i] != c->d_J) ? J[i] : nullptr;
        s9[i].args.sc = sc ? sc[i] : nullptr;
        if (2 * (size_t)s3[i].blocks > c->red_elems || (size_t)s6[i].blocks > c->red_elems ||
            (size_t)s2[i].blocks > c->red_elems) {
            set_error("context %d: reduction buffer too small", i);
            return DFTG_ERR_STATE;
        }
    }
    // device layout: counters + done flags, error flag, prefix arrays, argument records
    const size_t off_err = sizeof(int) * ((size_t)kCtlInts + n);
    const size_t off_self = align16(off_err + sizeof(int));
    const size_t off_prefix = align16(off_self + sizeof(int) * (size_t)(n + 1));
    const size_t prefix_bytes = sizeof(int) * (size_t)kNumSteps * (n + 1);
    const size_t rec[kNumSteps] = {sizeof(SlicePArgs), sizeof(DensTcArgs), sizeof(SumsArgs), sizeof(LdaArgs),
                                   sizeof(MpArgs),     sizeof(VcbArgs),    sizeof(GoArgs),   sizeof(CexpArgs),
                                   sizeof(CtArgs),     sizeof(RedArgs)};
    size_t off_args[kNumSteps];
    size_t total = align16(off_prefix + prefix_bytes);
    for (int st = 0; st < kNumSteps; ++st) {
        off_args[st] = total;
        total = align16(total + rec[st] * n);
    }
    BatchPlan *bp = new (std::nothrow) BatchPlan();
    if (!bp) { set_error("host allocation failed"); return DFTG_ERR_NOMEM; }
    bp->nmol = n;
    bp->device = ctx[0]->device;
    bp->lmax = lmax;
    cudaError_t e = cudaDeviceGetAttribute(&bp->nsm, cudaDevAttrMultiProcessorCount, bp->device);
    if (e == cudaSuccess) e = cudaMalloc(&bp->d_mem, total);
    int least = 0, greatest = 0;
    if (e == cudaSuccess) e = cudaDeviceGetStreamPriorityRange(&least, &greatest);
    if (e == cudaSuccess) e = cudaStreamCreateWithPriority(&bp->aux, cudaStreamNonBlocking, greatest);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bp->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&bp->ev_join, cudaEventDisableTiming);
    if (e != cudaSuccess) {
        batch_plan_free(bp);
        return cuda_fail(e, "batch plan", __FILE__, __LINE__);
    }
    unsigned char *base = static_cast<unsigned char *>(bp->d_mem);
    bp->d_heads = reinterpret_cast<int *>(base);
    bp->d_done = bp->d_heads + kCtlInts;
    bp->d_err = reinterpret_cast<int *>(base + off_err);
    bp->zero_bytes = off_err;
    for (int i = 0; i < n; ++i) s2[i].args.done = bp->d_done + i;

    std::vector<unsigned char> h(total, 0);
    int *hself = reinterpret_cast<int *>(h.data() + off_self);
    for (int i = 0; i <= n; ++i) hself[i] = i > 0 ? 1 : 0;
    bp->d_self_prefix = reinterpret_cast<const int *>(base + off_self);
    int *hp = reinterpret_cast<int *>(h.data() + off_prefix);
    auto fill = [&](int st, auto &steps) {
        int *pre = hp + (size_t)st * (n + 1);
        pre[0] = 0;
        for (int i = 0; i < n; ++i) {
            pre[i + 1] = pre[i] + steps[i].blocks;
            bp->smem[st] = std::max(bp->smem[st], steps[i].smem);
            std::memcpy(h.data() + off_args[st] + rec[st] * i, &steps[i].args, rec[st]);
        }
        GroupQueue &q = bp->q[st];
        q.prefix = reinterpret_cast<const int *>(base + off_prefix) + (size_t)st * (n + 1);
        q.nmol = n;
        q.nitems = pre[n];
        q.take = kTake[st];
        q.head = bp->d_heads + st;
        bp->args[st] = base + off_args[st];
    };
    fill(kStSliceP, s0);
    fill(kStDensity, s1);
    fill(kStSums, s2);
    fill(kStLda, s3);
    fill(kStMultipole, s4);
    fill(kStVcb, s5);
    fill(kStGather, s6);
    fill(kStCexp, s7);
    fill(kStContract, s8);
    fill(kStReduce, s9);
    // one counter serves both item ranges of the fused atom-sum + point launch
    bp->q[kStSums].head = bp->q[kStLda].head;
    bp->q[kStSums].take = bp->q[kStLda].take;
    e = cudaSetDevice(bp->device);
    if (e == cudaSuccess) e = cudaMemcpy(bp->d_mem, h.data(), total, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        batch_plan_free(bp);
        return cuda_fail(e, "batch plan copy", __FILE__, __LINE__);
    }
    *out = bp;
    return DFTG_OK;
}

// the batch's launches on st; sums_lda_only: the counters and the fused
// atom-sum + point launch alone (the bounded-wait self-test)
int batch_plan_enqueue(const BatchPlan *bp, cudaStream_t st, int stall_mol, unsigned long long limit_ns,
                       bool sums_lda_only)
{
    const int nsm = bp->nsm, dev = bp->device;
    DFTG_CUDA(cudaMemsetAsync(bp->d_heads, 0, bp->zero_bytes, st));
    const SumsLdaCtl ctl{bp->q[kStLda].head, bp->d_done, bp->d_err, limit_ns, stall_mol};
    if (sums_lda_only) {
        // the self-test: one point item of molecule 0, which waits for a flag
        // that nothing sets (no atom-sum items run)
        GroupQueue qs = bp->q[kStSums], ql = bp->q[kStLda];
        qs.nitems = 0;
        ql.prefix = bp->d_self_prefix;
        ql.nitems = 1;
        ql.take = 1;
        return group_sums_lda(static_cast<const SumsArgs *>(bp->args[kStSums]), qs,
                              static_cast<const LdaArgs *>(bp->args[kStLda]), ql, ctl, nsm, st);
    }
    DFTG_TRY_L(group_slice_P(static_cast<const SlicePArgs *>(bp->args[kStSliceP]), bp->q[kStSliceP], nsm, st));
    DFTG_TRY_L(group_density_tc(static_cast<const DensTcArgs *>(bp->args[kStDensity]), bp->q[kStDensity],
                                bp->smem[kStDensity], dev, nsm, st));
    // with no atom-sum items the point kernel and the Hartree steps are
    // independent (the density launch corrected rho and wrote the rho w_becke
    // planes): the Hartree steps run on the greatest-priority branch beside it
    const bool fork = bp->q[kStSums].nitems == 0;
    const cudaStream_t sh = fork ? bp->aux : st;
    if (fork) {
        DFTG_CUDA(cudaEventRecord(bp->ev_fork, st));
        DFTG_CUDA(cudaStreamWaitEvent(bp->aux, bp->ev_fork, 0));
    }
    if (bp->q[kStSums].nitems + bp->q[kStLda].nitems > 0)
        DFTG_TRY_L(group_sums_lda(static_cast<const SumsArgs *>(bp->args[kStSums]), bp->q[kStSums],
                                  static_cast<const LdaArgs *>(bp->args[kStLda]), bp->q[kStLda], ctl, nsm, st));
    DFTG_TRY_L(group_multipole(static_cast<const MpArgs *>(bp->args[kStMultipole]), bp->q[kStMultipole],
                               bp->smem[kStMultipole], dev, nsm, sh));
    if (bp->q[kStVcb].nitems > 0)
        DFTG_TRY_L(group_vcross_bins(static_cast<const VcbArgs *>(bp->args[kStVcb]), bp->q[kStVcb], bp->lmax,
                                     bp->smem[kStVcb], nsm, sh));
    DFTG_TRY_L(group_gather_own(static_cast<const GoArgs *>(bp->args[kStGather]), bp->q[kStGather],
                                bp->smem[kStGather], dev, nsm, sh));
    if (fork) {
        DFTG_CUDA(cudaEventRecord(bp->ev_join, bp->aux));
        DFTG_CUDA(cudaStreamWaitEvent(st, bp->ev_join, 0));
    }
    DFTG_TRY_L(group_cexp(static_cast<const CexpArgs *>(bp->args[kStCexp]), bp->q[kStCexp], nsm, st));
    DFTG_TRY_L(group_contract_tc(static_cast<const CtArgs *>(bp->args[kStContract]), bp->q[kStContract],
                                 bp->smem[kStContract], dev, nsm, st));
    return group_contract_reduce(static_cast<const RedArgs *>(bp->args[kStReduce]), bp->q[kStReduce], nsm, st);
}

// the error flag of the batch's bounded waits (read and cleared; st synchronised)
int batch_plan_take_error(const BatchPlan *bp, cudaStream_t st, int *code)
{
    DFTG_CUDA(cudaStreamSynchronize(st));
    DFTG_CUDA(cudaMemcpy(code, bp->d_err, sizeof(int), cudaMemcpyDeviceToHost));
    if (*code) DFTG_CUDA(cudaMemset(bp->d_err, 0, sizeof(int)));
    return DFTG_OK;
}

}  // namespace dftg
