// fau_kernels.h -- launch interface between the host runtime and the kernels.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include "../../include/fau_gpu.h"

namespace fau {

// An NVTX range over a host phase (an entry point of the C ABI): named in a profiler's timeline
// (nsys, ncu's range filter); without one attached, push and pop return at once.
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange&) = delete;
    NvtxRange& operator=(const NvtxRange&) = delete;
};

struct DevSys;

// Arguments of the persistent chain kernel; one CTA per entry of `sys`.
struct ChainArgs {
    DevSys* const* sys;          // device array of device DevSys pointers
    const uint32_t* sys_ids;     // RNG stream id per CTA (NULL: blockIdx.x)
    const long long* n_moves;    // moves per CTA (NULL: `moves`)
    long long moves;
    // host-fed proposal mode
    const fau_proposal* props;   // device proposal stream
    const long long* prop_off;   // first proposal per CTA (NULL: 0)
    uint8_t* acc_out;            // optional per-move outputs (indexed like props)
    double* du_out;
    fau_trial_result* detail;
    // device RNG mode
    uint64_t seed;
    unsigned long long counter_base;
    const unsigned long long* counters; // per CTA first counter (NULL: counter_base)
    double dp, dprot;
    const double* dp_sys;        // per CTA dp / dprot (NULL: dp, dprot)
    const double* dprot_sys;
    const uint8_t* molecular;    // per CTA: 1 -> moltransrot moves, 0 -> transrot
    // evaluate-only mode (one move, one CTA): no Metropolis, no commit; the trial is
    // written to `pending` and its Q(k) change to `pending_dq` for a later commit
    struct PlainMove* pending;
    double2* pending_dq;
    // optional per-CTA phase timers (clock64 cycles, kPhaseSlots per CTA) for profiling
    unsigned long long* phase_cycles;
    // > 0: a CTA ends its chain at the first move boundary after this many ns of its own
    // (globaltimer); G.consumed then holds the moves done
    unsigned long long time_budget_ns;
    // 1: after its last move each chain of the pipelined kernel evaluates one more (its next
    // proposal) on the final state without deciding it and leaves it for fast_audit_kernel
    int audit;
};
constexpr int kPhaseSlots = 17;     // chain kernel (last slot: move count)
constexpr int kFastPhaseSlots = 24; // pipelined kernel (the per-CTA stride of phase_cycles for both)

// One trial move held for a later commit (plain FP64 form and evaluate-only mode).
struct PlainMove {
    int kind, first, m, group;
    int count_move, pad; // 1: the commit also counts the move (plain form); 0: already counted
    double xn[32][3];
    double cm_new[3];
    double dM[3];
    double du;
};

constexpr int kTotalPairBlocks = 4096;
constexpr int kTotalMiscBlocks = 1024;
constexpr int kTotalPartials = kTotalPairBlocks + 2 * kTotalMiscBlocks;

size_t chain_smem_bytes(int K, int nc);
int chain_max_k(int threads);
cudaError_t prepare_chain(int K, int nc, int threads, bool philox);
cudaError_t launch_chain(const ChainArgs& a, int nblocks, int K, int nc, int threads, bool philox, cudaStream_t st);
// per (CTA size, proposal source) instantiations of the chain kernel
cudaError_t chain_dispatch_128_host(const ChainArgs&, int, int, int, cudaStream_t, bool);
cudaError_t chain_dispatch_128_ph(const ChainArgs&, int, int, int, cudaStream_t, bool);
cudaError_t chain_dispatch_256_host(const ChainArgs&, int, int, int, cudaStream_t, bool);
cudaError_t chain_dispatch_256_ph(const ChainArgs&, int, int, int, cudaStream_t, bool);
// pipelined molecular-move kernel (device proposals; 256 threads: 1 preparing + 7 compute warps)
cudaError_t mol_dispatch_256(const ChainArgs&, int, int, int, cudaStream_t, bool);
cudaError_t mol_dispatch_256_host(const ChainArgs&, int, int, int, cudaStream_t, bool); // host proposals
cudaError_t mol_dispatch_512(const ChainArgs&, int, int, int, cudaStream_t, bool);      // 1 + 15 warps, device proposals
int mol_minb(int nblocks); // CTAs per SM the molecular kernel's registers are sized for
size_t mol_smem_bytes_total(int K, int nc);
// pipelined chain kernel (single-atom moves only): 1 producer warp + `warps` compute warps;
// k-vector components up to kFastMaxNc (8-bit phase-table indices)
constexpr int kFastMaxNc = 40;
size_t fast_smem_bytes_total(int K, int nc, int nt);
// the FP64 audit of the pipelined kernel's probe moves (one CTA per system of `sys`)
cudaError_t launch_fast_audit(DevSys* const* sys, int n, cudaStream_t st);
// the FP64 audit of the molecular and chain kernels' probe moves (one CTA per system of `sys`)
cudaError_t launch_probe_audit(DevSys* const* sys, int n, cudaStream_t st);
// occ: a system of the launch is flagged SYS_OCC.  Then 4 and 8 compute warps run the instance
// holding every staging body, each CTA choosing by its system; otherwise the instance holding
// only the whole-cell body (the same code for those systems, without the register pressure of
// the occupied-slot bodies, which spill in the combined kernel).  2 compute warps: whole cells.
// 8 compute warps take device (Philox) proposals only.
cudaError_t prepare_fast(int K, int nc, int nt, int warps, bool philox, bool occ);
cudaError_t launch_fast(const ChainArgs& a, int nblocks, int K, int nc, int nt, int warps, bool philox, bool occ,
                        cudaStream_t st);
// the occupied-slot rules, fixed per system when it is made: any cell list stages its occupied
// slots only (from 0.2 particles a cell in dilute salt to tens in dense primitive models); with
// more particles than cells the stencil's cells are spread over all compute warps, otherwise
// they sit with the first warps' lanes, so that the other warps skip the pair rounds
inline bool fast_occupied_slots(bool cells) { return cells; }
inline bool fast_spread_cells(bool cells, int n, int ncell) { return cells && n > ncell; }
cudaError_t fast_dispatch_2_host(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_2_ph(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_4_host(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_4_ph(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_8_ph(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_4_host_sparse(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_4_ph_sparse(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
cudaError_t fast_dispatch_8_ph_sparse(const ChainArgs&, int, int, int, int, cudaStream_t, bool);
// cells: the system's groups are all atomic and it has a cell list (O(N x neighbours) pair sum)
cudaError_t launch_total(const DevSys* dsys, int n, int K, double* d_out, int* d_flags, cudaStream_t st,
                         bool cells = false);
cudaError_t launch_q_rebuild(const DevSys* dsys, int K, double2* out, cudaStream_t st);
cudaError_t launch_fold_q(DevSys* dsys, int K, cudaStream_t st); // pending Q(k) changes into the master
cudaError_t launch_plain_du(const DevSys* dsys, const PlainMove* pm, int n, int K, double2* dq, double* out,
                            int* flags, cudaStream_t st);
cudaError_t launch_plain_commit(DevSys* dsys, const PlainMove* pm, int K, const double2* dq, cudaStream_t st);
// FP64 replica chains (systems made with FAU_PREC_FP64; single-atom and rigid-molecule moves,
// 128-thread CTAs): the plain FP64 form's arithmetic as a persistent chain, one CTA per system;
// K and n_groups the largest of the launch's systems
size_t fp64_smem_bytes(int K, int n_groups);
cudaError_t prepare_fp64(int K, int n_groups, bool philox);
cudaError_t launch_fp64(const ChainArgs& a, int nblocks, int K, int n_groups, bool philox, cudaStream_t st);

} // namespace fau
