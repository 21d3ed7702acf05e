// fau_batch.cu -- many independent systems (replicas, parallel-tempering
// walkers, served jobs) advanced by one chain-kernel launch per block of
// moves, with device-side parallel-tempering swaps between blocks; the whole
// sequence is captured once into a CUDA graph and replayed.
//
// Parallel tempering follows the semantics of ParallelTempering
// (src/move.cpp:844-970): odd/even partner pairs (OddEvenPartner::generate,
// src/mpicontroller.cpp:69-83), acceptance on the sum of each walker's energy
// change in its own kT.  Exchanging configurations between two temperatures is
// done by exchanging the temperatures (the beta multiplier of each system).
#include "fau_dev.cuh"
#include "fau_kernels.h"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

using namespace fau;

// opaque handle layouts shared with fau_capi.cu
struct fau_ctx;
extern "C" int fau_internal_ctx_stream(fau_ctx* c, cudaStream_t* st, int* device);
extern "C" int fau_internal_sys_view(fau_sys* s, fau_ctx** ctx, DevSys** d, int* K, int* n, int* n_groups,
                                     int* molecular_only, double* t_ref, int* knc);
extern "C" int fau_internal_fail(int code, const char* msg);
extern "C" int fau_internal_ctx_scratch(fau_ctx* c, size_t bytes, void** out);
extern "C" int fau_internal_sys_all_atomic(const fau_sys* s);
extern "C" int fau_internal_sys_classes(const fau_sys* s);
extern "C" int fau_internal_sys_maxe(const fau_sys* s);
extern "C" int fau_internal_sys_fp64(const fau_sys* s);
extern "C" int fau_internal_sys_occ(const fau_sys* s);
extern "C" int fau_internal_sys_regrow(fau_sys* s);
cudaError_t fau_internal_sampler_launch(fau_sampler* s, DevSys* const* d_sys, int n, const int* d_slots, int max_n,
                                        cudaStream_t st);
int fau_internal_sampler_slots(const fau_sampler* s);
fau_ctx* fau_internal_sampler_ctx(const fau_sampler* s);

// FAU_ERR_CUDA with the failing call and the runtime's name and text of the error (a fault in
// one of the batch's kernels surfaces at the first synchronising call after the graph)
static int fau_internal_fail_cuda(cudaError_t e, const char* what)
{
    const std::string msg = std::string(what) + " failed: " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fau_internal_fail(FAU_ERR_CUDA, msg.c_str());
}

namespace {

// per-system summary gathered after a run
struct SysSummary {
    unsigned long long moves, accepted, pair_evals, k_updates, cycles;
    double energy, beta_scale;
    int err, pad;
    long long consumed; // proposals performed by the system's last chain launch
    double audit_scaled, audit_rel;
    unsigned long long audit_samples;
};

__global__ void gather_kernel(DevSys* const* sys, int n, SysSummary* out)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const DevSys& S = *sys[i];
        out[i] = {S.moves,      S.accepted, S.pair_evals, S.k_updates,        S.cycles,        sys_energy(S),
                  S.beta_scale, S.err,      0,            S.consumed,         S.audit_scaled_max, S.audit_rel_max,
                  S.audit_samples};
    }
}

// One parallel-tempering exchange step over the temperature ladder.
// slot_sys[s]: system holding temperature slot s; T[s]: slot temperatures;
// Tref[i]: temperature system i's parameters were built for (its kT unit).
// Energies are converted to absolute units (kT_ref * T_ref) and pairs
// (s, s+1) with s = parity, parity + 2, ... are exchanged as metropolisCriterion
// (src/montecarlo.cpp:17-34) decides on dU = -x, x = (1/T_s - 1/T_{s+1}) (E_a - E_b):
// accept when u <= exp(x) (always for x >= 0; never for a NaN).  The optional logs
// receive each system's running energy at the round and the slot order after it.
__global__ void pt_swap_kernel(DevSys* const* sys, int n, int* slot_sys, const double* T, const double* Tref,
                               uint64_t seed, unsigned long long round, unsigned long long* stats,
                               double* energy_log, int* slots_log)
{
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    if (energy_log)
        for (int i = 0; i < n; i++) energy_log[i] = sys_energy(*sys[i]);
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const U4 r0 = philox({(uint32_t)round, (uint32_t)(round >> 32), 0xFFFFFFFFu, 7u}, k0, k1);
    const int parity = r0.x & 1;
    for (int s = parity; s + 1 < n; s += 2) {
        const int a = slot_sys[s], b = slot_sys[s + 1];
        const double Ea = sys_energy(*sys[a]) * Tref[a];
        const double Eb = sys_energy(*sys[b]) * Tref[b];
        const double x = (1.0 / T[s] - 1.0 / T[s + 1]) * (Ea - Eb);
        const U4 r = philox({(uint32_t)round, (uint32_t)(round >> 32), (uint32_t)s, 8u}, k0, k1);
        const double u = u01_53(r.x, r.y);
        stats[0]++;
        bool acc = false;
        if (x >= 0.0) acc = true;
        else if (!isnan(x)) acc = u <= exp(x);
        if (acc) {
            stats[1]++;
            slot_sys[s] = b;
            slot_sys[s + 1] = a;
            sys[a]->beta_scale = Tref[a] / T[s + 1];
            sys[b]->beta_scale = Tref[b] / T[s];
        }
    }
    if (slots_log)
        for (int s = 0; s < n; s++) slots_log[s] = slot_sys[s];
}

// the pipelined kernel writes each move's energy change as a packed float-float pair
// {hi, lo}; one CTA per system turns its range into FP64 values in place
__global__ void unpack_du_kernel(double* du, const long long* off, const long long* nm)
{
    const long long o = off[blockIdx.x], n = nm[blockIdx.x];
    float2* p = reinterpret_cast<float2*>(du);
    for (long long m = threadIdx.x; m < n; m += blockDim.x) {
        const float2 v = p[o + m];
        du[o + m] = (double)v.x + (double)v.y;
    }
}

// each parallel-tempering run starts with every system at its own temperature
__global__ void reset_beta_kernel(DevSys* const* sys, int n)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) sys[i]->beta_scale = 1.0;
}

// Philox4x32-10 on the host (Salmon, Moraes, Dror & Shaw, SC'11, published constants), the same
// generator the device draws its proposals and swap decisions from
void philox_host(uint32_t c[4], uint32_t k0, uint32_t k1)
{
    for (int r = 0; r < 10; r++) {
        const unsigned long long p0 = 0xD2511F53ull * c[0], p1 = 0xCD9E8D57ull * c[2];
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c[1] ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c[3] ^ k1;
        c[0] = n0;
        c[1] = (uint32_t)p1;
        c[2] = n2;
        c[3] = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}
double u01_53_host(uint32_t a, uint32_t b)
{
    return (double)((((unsigned long long)(a >> 5)) << 26) | (b >> 6)) * (1.0 / 9007199254740992.0);
}

} // namespace

extern "C" double fau_internal_sys_volume(const fau_sys* s);

namespace {
const char* const kFp64Mixed = "a batch holds FP64 systems (FAU_PREC_FP64) only or none";
const char* const kFp64Form = "FP64 chains run systems without a finite maxenergy";

// 1: every system of the batch is an FP64 system, 0: none is; -1: both kinds; -2: an FP64 system
// the FP64 chain kernel does not run (a finite maxenergy)
int fp64_batch(fau_sys* const* systems, int n)
{
    int k = 0;
    for (int i = 0; i < n; i++) k += fau_internal_sys_fp64(systems[i]);
    if (k == 0) return 0;
    if (k != n) return -1;
    for (int i = 0; i < n; i++)
        if (fau_internal_sys_maxe(systems[i])) return -2;
    return 1;
}

// the largest group count of the batch (the FP64 kernel's per-group GroupCutoff flags)
int max_groups(fau_sys* const* systems, int n)
{
    int g = 0;
    for (int i = 0; i < n; i++) {
        fau_ctx* c2;
        DevSys* dd;
        int K, np, ng, mo, knc;
        double tr;
        fau_internal_sys_view(systems[i], &c2, &dd, &K, &np, &ng, &mo, &tr, &knc);
        g = std::max(g, ng);
    }
    return g;
}
} // namespace

// NPT blocks: each block's moves through fau_run_batch (one graph launch), then one VolumeMove
// per system (VolumeMove::_move and setNewVolume, src/move.cpp:994-1006, decided as
// fau_volume_move decides it)
static int run_volume_blocks(fau_ctx* ctx, fau_sys* const* systems, int n, const fau_batch_params* P,
                             fau_batch_stats* stats)
{
    const long long iv = P->volume_interval_moves;
    fau_batch_stats S{};
    std::vector<uint64_t> ctr(n), cyc(n), cyc_b(n);
    const unsigned long long key = P->seed ^ 0x5DEECE66DULL;
    for (int b = 0; b < P->n_volume_blocks; b++) {
        fau_batch_params sub = *P;
        sub.volume_interval_moves = 0;
        sub.n_volume_blocks = 0;
        sub.moves = iv;
        sub.moves_out = nullptr;
        sub.cycles_out = P->cycles_out ? cyc_b.data() : nullptr;
        for (int i = 0; i < n; i++) ctr[i] = (P->counters ? P->counters[i] : 0ull) + (uint64_t)b * (uint64_t)iv;
        sub.counters = ctr.data();
        fau_batch_stats sb{};
        int rc = fau_run_batch(ctx, systems, n, &sub, &sb);
        if (rc != FAU_OK) return rc;
        S.moves += sb.moves;
        S.accepted += sb.accepted;
        S.pair_evals += sb.pair_evals;
        S.k_updates += sb.k_updates;
        S.device_ms += sb.device_ms;
        S.du_err_scaled_max = std::max(S.du_err_scaled_max, sb.du_err_scaled_max);
        S.du_err_rel_max = std::max(S.du_err_rel_max, sb.du_err_rel_max);
        S.du_err_samples += sb.du_err_samples;
        if (P->cycles_out)
            for (int i = 0; i < n; i++) cyc[i] += cyc_b[i];
        if (!(P->volume_dv > 0.0)) continue; // VolumeMove::_move: no change without a displacement
        for (int i = 0; i < n; i++) {
            const uint32_t stream = P->streams ? P->streams[i] : (uint32_t)i;
            const unsigned long long v =
                ((P->counters ? P->counters[i] : 0ull) + P->counter_base) / (unsigned long long)iv + (unsigned long long)b;
            uint32_t w[4] = {(uint32_t)v, (uint32_t)(v >> 32), stream, 9u};
            philox_host(w, (uint32_t)key, (uint32_t)(key >> 32));
            const double ua = u01_53_host(w[0], w[1]), ub = u01_53_host(w[2], w[3]);
            const double V = fau_internal_sys_volume(systems[i]);
            const double nv = std::exp(std::log(V) + (ua - 0.5) * P->volume_dv);
            fau_trial_result tr{};
            if ((rc = fau_volume_move(systems[i], nv, P->volume_method, ub, &tr)) != FAU_OK) return rc;
            S.moves += 1;
            S.volume_attempted += 1;
            if (tr.accepted) {
                S.accepted += 1;
                S.volume_accepted += 1;
            }
        }
    }
    if (P->moves_out)
        for (int i = 0; i < n; i++)
            P->moves_out[i] = (int64_t)P->n_volume_blocks * (iv + (P->volume_dv > 0.0 ? 1 : 0));
    if (P->cycles_out)
        for (int i = 0; i < n; i++) P->cycles_out[i] = cyc[i];
    if (stats) *stats = S;
    return FAU_OK;
}

extern "C" int fau_run_batch(fau_ctx* ctx, fau_sys* const* systems, int n, const fau_batch_params* P,
                             fau_batch_stats* stats)
{
    const NvtxRange nvtx_range("fau_run_batch");
    if (!ctx || !systems || !P || n < 1) return fau_internal_fail(FAU_ERR_ARG, "invalid batch arguments");
    cudaStream_t st;
    int device;
    fau_internal_ctx_stream(ctx, &st, &device);
    if (cudaSetDevice(device) != cudaSuccess) return fau_internal_fail(FAU_ERR_CUDA, "cudaSetDevice failed");
    const bool pt = P->swap_interval_moves > 0 && P->n_swap_blocks > 0;
    if (pt && !P->temperatures) return fau_internal_fail(FAU_ERR_ARG, "parallel tempering needs temperatures");
    // blocks of moves: PT swap blocks, or sample blocks of a device sampler, or one block
    fau_sampler* smp = P->sampler;
    if (smp && fau_internal_sampler_ctx(smp) != ctx) return fau_internal_fail(FAU_ERR_ARG, "sampler from another context");
    const bool sblocks = !pt && smp && P->sample_interval_moves > 0 && P->n_sample_blocks > 0;
    if (sblocks && P->moves_per_system)
        return fau_internal_fail(FAU_ERR_ARG, "sample blocks take a common move count (moves_per_system must be NULL)");
    const bool blocked = pt || sblocks;
    const long long blk_moves = pt ? P->swap_interval_moves : (sblocks ? P->sample_interval_moves : 0);
    const int nblk = pt ? P->n_swap_blocks : (sblocks ? P->n_sample_blocks : 1);
    // parallel tempering with a block length per walker (moves_per_system: e.g. 1,000 sweeps each)
    const bool pt_lens = pt && P->moves_per_system;
    const bool pt_log = pt && (P->swap_slots_out || P->swap_energy_out);
    if (!(P->dp >= 0.0)) return fau_internal_fail(FAU_ERR_ARG, "dp must be >= 0");
    if (P->volume_interval_moves != 0 || P->n_volume_blocks != 0) {
        if (P->volume_interval_moves <= 0 || P->n_volume_blocks <= 0)
            return fau_internal_fail(FAU_ERR_ARG, "volume blocks need volume_interval_moves > 0 and n_volume_blocks > 0");
        if (pt || smp || P->time_budget_ns || P->moves_per_system)
            return fau_internal_fail(FAU_ERR_ARG, "volume blocks take one move count and no PT, sampler or time budget");
        if (!(P->volume_dv >= 0.0) || !std::isfinite(P->volume_dv))
            return fau_internal_fail(FAU_ERR_ARG, "volume_dv must be finite and >= 0");
        if (P->volume_method < FAU_VOLUME_ISOTROPIC || P->volume_method > FAU_VOLUME_ISOCHORIC)
            return fau_internal_fail(FAU_ERR_ARG, "unknown volume scaling method");
        return run_volume_blocks(ctx, systems, n, P, stats);
    }

    std::vector<DevSys*> dsys(n);
    std::vector<long long> nm(n);
    std::vector<uint32_t> ids(n);
    std::vector<uint8_t> mol(n);
    std::vector<double> tref(n, 1.0);
    for (int i = 0; i < n; i++) {
        fau_ctx* c2;
        int K, np, ng, mo, knc;
        fau_internal_sys_view(systems[i], &c2, &dsys[i], &K, &np, &ng, &mo, &tref[i], &knc);
        if (c2 != ctx) return fau_internal_fail(FAU_ERR_ARG, "system from another context");
        nm[i] = P->moves_per_system ? P->moves_per_system[i] : P->moves;
        if (nm[i] < 0) return fau_internal_fail(FAU_ERR_ARG, "negative move count");
        ids[i] = P->streams ? P->streams[i] : (uint32_t)i;
        mol[i] = (uint8_t)mo;
        if (pt) tref[i] = P->temperatures[i];
    }
    // systems made with FAU_PREC_FP64 run in the FP64 chain kernel: a batch holds FP64 systems only
    // or none, without a finite maxenergy
    const int f64 = fp64_batch(systems, n);
    const int g64 = f64 > 0 ? max_groups(systems, n) : 0;
    if (f64 < 0) return f64 == -1 ? fau_internal_fail(FAU_ERR_ARG, kFp64Mixed) : fau_internal_fail(FAU_ERR_ARG, kFp64Form);
    // kernel choice: threads 0, 96, 160 or 288 -> the pipelined kernel (1 producer + 4, 2, 4 or 8
    // compute warps) for every system whose device proposals are single-atom moves (the others run
    // in the 256-thread chain kernel); 128 or 256 -> the chain kernel of that size for all systems;
    // 512 -> as 0, with molecular-move systems in 512-thread CTAs of the pipelined molecular kernel
    // (1 preparing + 15 compute warps, one CTA an SM: each chain's moves take less time)
    const int req = P->threads;
    if (req != 0 && req != 96 && req != 128 && req != 160 && req != 256 && req != 288 && req != 512)
        return fau_internal_fail(FAU_ERR_ARG, "threads must be 0, 96, 128, 160, 256, 288 or 512");
    bool mol512 = req == 512;
    const bool use_fast = req == 0 || req == 96 || req == 160 || req == 288 || mol512;
    const int threads = use_fast ? 256 : req; // molecular moves: 256-thread chain CTAs measured fastest
    int fwarps = req == 96 ? 2 : (req == 288 ? 8 : 4);
    std::vector<uint8_t> fast(n, 0);
    for (int i = 0; i < n; i++) {
        fau_ctx* c2;
        int K, np, ng, mo, knc;
        double tr;
        DevSys* dd;
        fau_internal_sys_view(systems[i], &c2, &dd, &K, &np, &ng, &mo, &tr, &knc);
        // a finite maxenergy: the chain kernel (the only one that forms each state's term sums)
        fast[i] = !f64 && use_fast && !mol[i] && knc <= kFastMaxNc && !fau_internal_sys_maxe(systems[i]);
    }
    std::vector<int> order;   // kernel order: pipelined-kernel systems first
    order.reserve(n);
    for (int i = 0; i < n; i++)
        if (fast[i]) order.push_back(i);
    const int nfast = (int)order.size();
    for (int i = 0; i < n; i++)
        if (!fast[i]) order.push_back(i);
    const int nexact = n - nfast;
    // within each kernel, chains in descending order of their work (moves x particles): the CTAs
    // are handed to the SMs in index order, so the longest chains start first, one to an SM while
    // SMs remain, and the short ones fill in beside them (results depend only on each system's
    // seed, stream and counter, never on this order)
    {
        std::vector<double> cost(n);
        for (int i = 0; i < n; i++) {
            fau_ctx* c2;
            int K, np, ng, mo, knc;
            double tr;
            DevSys* dd;
            fau_internal_sys_view(systems[i], &c2, &dd, &K, &np, &ng, &mo, &tr, &knc);
            const double len = blocked && !pt_lens ? (double)blk_moves : (double)nm[i];
            cost[i] = len * (double)(np + K);
        }
        auto by_cost = [&](int x, int y) { return cost[x] > cost[y]; };
        std::stable_sort(order.begin(), order.begin() + nfast, by_cost);
        std::stable_sort(order.begin() + nfast, order.end(), by_cost);
    }
    int Kf = 0, ncf = 0, ntf = 1, Ke = 0, nce = 0;
    bool occf = false; // a pipelined system stages occupied slots: the instance holding that body
    for (int r = 0; r < n; r++) {
        int K, np, ng, mo, knc;
        fau_ctx* c2;
        DevSys* dd;
        double tr;
        fau_internal_sys_view(systems[order[r]], &c2, &dd, &K, &np, &ng, &mo, &tr, &knc);
        if (r < nfast) {
            Kf = std::max(Kf, K);
            ncf = std::max(ncf, knc);
            ntf = std::max(ntf, fau_internal_sys_classes(systems[order[r]]));
            occf = occf || fau_internal_sys_occ(systems[order[r]]);
        }
        else {
            Ke = std::max(Ke, K);
            nce = std::max(nce, knc);
        }
    }
    if (f64 ? fp64_smem_bytes(Ke, g64) + 16384 > 227 * 1024
            : ((nexact && (Ke > chain_max_k(threads) || chain_smem_bytes(Ke, nce) + 16384 > 227 * 1024)) ||
               (nfast && fast_smem_bytes_total(Kf, ncf, ntf) > 227 * 1024)))
        return fau_internal_fail(FAU_ERR_ARG, "too many k-vectors (FP64 chains: k-vectors and groups) for the chain kernel");
    // molecular-move systems: the pipelined molecular kernel (preparation of the next move overlapped
    // with the current one) unless a chain-kernel size was requested; FAU_MOL_KERNEL=0 turns it off
    bool use_mol = !f64 && use_fast && nexact > 0;
    if (const char* mk = std::getenv("FAU_MOL_KERNEL"); mk && mk[0] == '0') use_mol = false;
    for (int r = nfast; r < n && use_mol; r++)
        if (!mol[order[r]] || fau_internal_sys_maxe(systems[order[r]])) use_mol = false;
    if (use_mol && mol_smem_bytes_total(Ke, nce) + (mol512 ? 36864 : 24576) > 227 * 1024) use_mol = false;
    // threads 0, molecular chains alone in the launch: 512-thread CTAs when every chain fits on the
    // GPU at once with one CTA an SM and no time budget applies (a chain's moves take 20-30 % less
    // time; with more chains than SMs four 256-thread CTAs an SM hold more work).  The width sets
    // the FP32 summation order, so a chain depends on it, as for the pipelined single-atom kernel.
    if (req == 0 && use_mol && nfast == 0 && P->time_budget_ns == 0 &&
        mol_smem_bytes_total(Ke, nce) + 36864 <= 227 * 1024) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sms = 0;
        if (nexact <= sms) mol512 = true;
    }
    // threads 0: the pipelined kernel's width for this launch.  When every chain fits on the GPU at
    // once in CTAs of 8 compute warps (two to an SM, shared memory allowing) each chain gets those:
    // its moves take less time, and a block (parallel tempering) lasts as long as its longest
    // chain.  More chains than that keep CTAs of 4, so that four chains share an SM; so do served
    // (time-budgeted) launches and launches beside the chain kernel.  One pipelined launch a block.
    if (req == 0 && nfast > 0 && nexact == 0 && P->time_budget_ns == 0) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sms = 0;
        const size_t per_cta = fast_smem_bytes_total(Kf, ncf, ntf) + 1024; // + the runtime's reserve
        const int per_sm = (int)std::min<size_t>(2, (size_t)228 * 1024 / per_cta);
        if (nfast <= per_sm * sms) fwarps = 8;
    }

    // device argument arrays (one allocation, freed at the end of the call)
    // every sub-buffer starts on a 16-byte boundary (8-byte fields inside)
    auto al = [](size_t x) { return (x + 15) & ~size_t(15); };
    const size_t off_sys = 0, off_nm = al(off_sys + sizeof(DevSys*) * n), off_ids = al(off_nm + 8 * n),
                 off_mol = al(off_ids + 4 * n), off_slot = al(off_mol + n), off_T = al(off_slot + 4 * n),
                 off_Tref = al(off_T + 8 * n), off_sum = al(off_Tref + 8 * n),
                 off_st = al(off_sum + sizeof(SysSummary) * n), off_ctr = al(off_st + 64),
                 off_ksys = al(off_ctr + 8 * n), off_knm = al(off_ksys + sizeof(DevSys*) * n),
                 off_kids = al(off_knm + 8 * n), off_kmol = al(off_kids + 4 * n), off_kctr = al(off_kmol + n),
                 off_kdp = al(off_kctr + 8 * n), off_kdr = al(off_kdp + 8 * n), off_sslot = al(off_kdr + 8 * n),
                 off_bctr = al(off_sslot + 4 * n), off_elog = al(off_bctr + 8 * (size_t)n * nblk),
                 off_slog = al(off_elog + (pt_log ? 8 * (size_t)n * nblk : 0)),
                 total = al(off_slog + (pt_log ? 4 * (size_t)n * nblk : 0));
    unsigned char* dbuf = nullptr;
    if (fau_internal_ctx_scratch(ctx, total, reinterpret_cast<void**>(&dbuf)) != FAU_OK)
        return fau_internal_fail(FAU_ERR_OOM, "batch argument allocation");
    std::vector<int> slot(n);
    for (int i = 0; i < n; i++) slot[i] = i;
    int rc = FAU_OK;
    cudaStream_t st2 = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    auto release2 = [&]() {
        if (st2) cudaStreamDestroy(st2);
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        st2 = nullptr;
        fork_ev = join_ev = nullptr;
    };
    auto cleanup = [&]() { release2(); }; // dbuf is the context's scratch
#define BTRY(x)                                                                 \
    do {                                                                        \
        const cudaError_t be_ = (x);                                            \
        if (be_ != cudaSuccess) {                                               \
            cleanup();                                                          \
            return fau_internal_fail_cuda(be_, "batch: " #x);                   \
        }                                                                       \
    } while (0)
    BTRY(cudaMemcpyAsync(dbuf + off_sys, dsys.data(), sizeof(DevSys*) * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_ids, ids.data(), 4 * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_mol, mol.data(), n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_slot, slot.data(), 4 * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemsetAsync(dbuf + off_st, 0, 64, st));
    if (pt) {
        BTRY(cudaMemcpyAsync(dbuf + off_T, P->temperatures, 8 * n, cudaMemcpyHostToDevice, st));
        BTRY(cudaMemcpyAsync(dbuf + off_Tref, tref.data(), 8 * n, cudaMemcpyHostToDevice, st));
    }
    int max_np = 0;
    if (smp) {
        const int ns = fau_internal_sampler_slots(smp);
        std::vector<int> sslot(n);
        for (int i = 0; i < n; i++) {
            sslot[i] = P->sample_slots ? P->sample_slots[i] : i % ns;
            if (sslot[i] < 0 || sslot[i] >= ns) {
                cleanup();
                return fau_internal_fail(FAU_ERR_ARG, "sample slot outside [0, n_slots)");
            }
            fau_ctx* c2;
            int K, np, ng, mo, knc;
            double tr;
            DevSys* dd;
            fau_internal_sys_view(systems[i], &c2, &dd, &K, &np, &ng, &mo, &tr, &knc);
            max_np = std::max(max_np, np);
        }
        BTRY(cudaMemcpyAsync(dbuf + off_sslot, sslot.data(), 4 * n, cudaMemcpyHostToDevice, st));
    }
    DevSys* const* d_sys = reinterpret_cast<DevSys* const*>(dbuf + off_sys);
    SysSummary* d_sum = reinterpret_cast<SysSummary*>(dbuf + off_sum);

    if (pt) reset_beta_kernel<<<(n + 127) / 128, 128, 0, st>>>(d_sys, n);
    // baseline counters
    std::vector<SysSummary> s0(n), s1(n);
    gather_kernel<<<(n + 127) / 128, 128, 0, st>>>(d_sys, n, d_sum);
    BTRY(cudaMemcpyAsync(s0.data(), d_sum, sizeof(SysSummary) * n, cudaMemcpyDeviceToHost, st));

    // per-CTA arguments in kernel order
    std::vector<DevSys*> ksys(n);
    std::vector<long long> knm(n);
    std::vector<uint32_t> kids(n);
    std::vector<uint8_t> kmol(n);
    std::vector<unsigned long long> kctr(n, 0);
    std::vector<double> kdp(n, P->dp), kdr(n, P->dprot);
    for (int r = 0; r < n; r++) {
        const int i = order[r];
        ksys[r] = dsys[i];
        knm[r] = nm[i];
        kids[r] = ids[i];
        kmol[r] = mol[i];
        if (P->counters) kctr[r] = P->counters[i];
        if (P->dp_per_system) kdp[r] = P->dp_per_system[i];
        if (P->dprot_per_system) kdr[r] = P->dprot_per_system[i];
        if (!(kdp[r] >= 0.0) || !(kdr[r] >= 0.0)) {
            cleanup();
            return fau_internal_fail(FAU_ERR_ARG, "dp and dprot must be >= 0");
        }
    }
    BTRY(cudaMemcpyAsync(dbuf + off_ksys, ksys.data(), sizeof(DevSys*) * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_knm, knm.data(), 8 * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_kids, kids.data(), 4 * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_kmol, kmol.data(), n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_kctr, kctr.data(), 8 * n, cudaMemcpyHostToDevice, st));
    // blocked launches: each block's first move counter per CTA (a walker's block b starts at
    // its counter + b times its own block length)
    std::vector<unsigned long long> bctr;
    if (blocked) {
        bctr.resize((size_t)n * nblk);
        for (int b = 0; b < nblk; b++)
            for (int r = 0; r < n; r++)
                bctr[(size_t)b * n + r] =
                    kctr[r] + (unsigned long long)b * (unsigned long long)(pt_lens ? knm[r] : blk_moves);
        BTRY(cudaMemcpyAsync(dbuf + off_bctr, bctr.data(), 8 * bctr.size(), cudaMemcpyHostToDevice, st));
    }
    BTRY(cudaMemcpyAsync(dbuf + off_kdp, kdp.data(), 8 * n, cudaMemcpyHostToDevice, st));
    BTRY(cudaMemcpyAsync(dbuf + off_kdr, kdr.data(), 8 * n, cudaMemcpyHostToDevice, st));
    ChainArgs a{};
    a.sys = reinterpret_cast<DevSys* const*>(dbuf + off_ksys);
    a.sys_ids = reinterpret_cast<const uint32_t*>(dbuf + off_kids);
    a.audit = P->no_audit ? 0 : 1;
    a.seed = P->seed;
    a.dp = P->dp;
    a.dprot = P->dprot;
    a.molecular = reinterpret_cast<const uint8_t*>(dbuf + off_kmol);
    a.dp_sys = reinterpret_cast<const double*>(dbuf + off_kdp);
    a.dprot_sys = reinterpret_cast<const double*>(dbuf + off_kdr);
    if (P->counters) a.counters = reinterpret_cast<const unsigned long long*>(dbuf + off_kctr);
    if (blocked) {
        a.n_moves = pt_lens ? reinterpret_cast<const long long*>(dbuf + off_knm) : nullptr;
        a.moves = blk_moves;
    }
    else {
        a.n_moves = reinterpret_cast<const long long*>(dbuf + off_knm);
        a.time_budget_ns = P->time_budget_ns; // chains may end early; moves_out reports how far
    }
    // the same arguments shifted to the chain-kernel systems
    ChainArgs ae = a;
    ae.sys = a.sys + nfast;
    ae.sys_ids = a.sys_ids + nfast;
    ae.molecular = a.molecular + nfast;
    ae.dp_sys = a.dp_sys + nfast;
    ae.dprot_sys = a.dprot_sys + nfast;
    if (a.counters) ae.counters = a.counters + nfast;
    if (a.n_moves) ae.n_moves = a.n_moves + nfast;
    // set the kernels' shared-memory attributes before the capture starts
    if (nexact)
        BTRY(f64       ? prepare_fp64(Ke, g64, true)
             : use_mol ? (mol512 ? mol_dispatch_512(ChainArgs{}, 0, Ke, nce, nullptr, true)
                                 : mol_dispatch_256(ChainArgs{}, 0, Ke, nce, nullptr, true))
                       : prepare_chain(Ke, nce, threads, true));
    if (nfast) BTRY(prepare_fast(Kf, ncf, ntf, fwarps, true, occf));
    if (nfast && nexact) {
        BTRY(cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking));
        BTRY(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        BTRY(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
    }
    // one block of moves: the pipelined kernel on `st`, the chain kernel on a forked stream
    auto launch_block = [&](int b) -> cudaError_t {
        if (blocked) { // this block's first counters (the CTA's counter + b block lengths)
            a.counters = reinterpret_cast<const unsigned long long*>(dbuf + off_bctr) + (size_t)b * n;
            ae.counters = a.counters + nfast;
        }
        a.counter_base = P->counter_base;
        ae.counter_base = P->counter_base;
        cudaError_t e = cudaSuccess;
        if (nfast && nexact) {
            if ((e = cudaEventRecord(fork_ev, st)) != cudaSuccess) return e;
            if ((e = cudaStreamWaitEvent(st2, fork_ev, 0)) != cudaSuccess) return e;
            if ((e = use_mol ? (mol512 ? mol_dispatch_512(ae, nexact, Ke, nce, st2, false)
                                       : mol_dispatch_256(ae, nexact, Ke, nce, st2, false))
                             : launch_chain(ae, nexact, Ke, nce, threads, true, st2)) != cudaSuccess)
                return e;
            if (a.audit && (e = launch_probe_audit(ae.sys, nexact, st2)) != cudaSuccess) return e;
            if ((e = cudaEventRecord(join_ev, st2)) != cudaSuccess) return e;
            if ((e = launch_fast(a, nfast, Kf, ncf, ntf, fwarps, true, occf, st)) != cudaSuccess) return e;
            if (a.audit && (e = launch_fast_audit(a.sys, nfast, st)) != cudaSuccess) return e;
            return cudaStreamWaitEvent(st, join_ev, 0);
        }
        if (nfast) {
            if ((e = launch_fast(a, nfast, Kf, ncf, ntf, fwarps, true, occf, st)) != cudaSuccess) return e;
            return a.audit ? launch_fast_audit(a.sys, nfast, st) : cudaSuccess;
        }
        if (f64) return launch_fp64(ae, nexact, Ke, g64, true, st);
        const cudaError_t e2 = use_mol ? (mol512 ? mol_dispatch_512(ae, nexact, Ke, nce, st, false)
                                                : mol_dispatch_256(ae, nexact, Ke, nce, st, false))
                                       : launch_chain(ae, nexact, Ke, nce, threads, true, st);
        if (e2 != cudaSuccess || !a.audit) return e2;
        return launch_probe_audit(ae.sys, nexact, st);
    };

    // profiling: FAU_PHASE_TIMING=1 prints the chain kernel's per-phase cycles to stderr
    unsigned long long* d_phase = nullptr;
    const char* pt_env = std::getenv("FAU_PHASE_TIMING");
    if (pt_env && pt_env[0] == '1') {
        if (cudaMalloc(&d_phase, sizeof(unsigned long long) * kFastPhaseSlots * n) == cudaSuccess) {
            cudaMemsetAsync(d_phase, 0, sizeof(unsigned long long) * kFastPhaseSlots * n, st);
            a.phase_cycles = d_phase;
            ae.phase_cycles = d_phase + (size_t)kFastPhaseSlots * nfast;
        }
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    BTRY(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
    for (int b = 0; b < nblk; b++) {
        if (launch_block(b) != cudaSuccess) {
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            cleanup();
            return fau_internal_fail(FAU_ERR_CUDA, "chain launch failed during capture");
        }
        if (pt)
            pt_swap_kernel<<<1, 1, 0, st>>>(d_sys, n, reinterpret_cast<int*>(dbuf + off_slot),
                                            reinterpret_cast<const double*>(dbuf + off_T),
                                            reinterpret_cast<const double*>(dbuf + off_Tref), P->seed ^ 0x5DEECE66DULL,
                                            P->counter_base / (P->swap_interval_moves ? P->swap_interval_moves : 1) + b,
                                            reinterpret_cast<unsigned long long*>(dbuf + off_st),
                                            pt_log ? reinterpret_cast<double*>(dbuf + off_elog) + (size_t)b * n : nullptr,
                                            pt_log ? reinterpret_cast<int*>(dbuf + off_slog) + (size_t)b * n : nullptr);
        if (smp && fau_internal_sampler_launch(smp, d_sys, n, reinterpret_cast<const int*>(dbuf + off_sslot), max_np,
                                               st) != cudaSuccess) {
            cudaStreamEndCapture(st, &graph);
            if (graph) cudaGraphDestroy(graph);
            cleanup();
            return fau_internal_fail(FAU_ERR_CUDA, "sampler launch failed during capture");
        }
    }
    BTRY(cudaStreamEndCapture(st, &graph));
    BTRY(cudaGraphInstantiate(&exec, graph, 0));
    BTRY(cudaEventRecord(e0, st));
    BTRY(cudaGraphLaunch(exec, st));
    BTRY(cudaEventRecord(e1, st));
    gather_kernel<<<(n + 127) / 128, 128, 0, st>>>(d_sys, n, d_sum);
    unsigned long long pst[8] = {0};
    BTRY(cudaMemcpyAsync(s1.data(), d_sum, sizeof(SysSummary) * n, cudaMemcpyDeviceToHost, st));
    BTRY(cudaMemcpyAsync(pst, dbuf + off_st, 64, cudaMemcpyDeviceToHost, st));
    if (pt_log && P->swap_energy_out)
        BTRY(cudaMemcpyAsync(P->swap_energy_out, dbuf + off_elog, 8 * (size_t)n * nblk, cudaMemcpyDeviceToHost, st));
    if (pt_log && P->swap_slots_out)
        BTRY(cudaMemcpyAsync(P->swap_slots_out, dbuf + off_slog, 4 * (size_t)n * nblk, cudaMemcpyDeviceToHost, st));
    const cudaError_t se = cudaStreamSynchronize(st);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaGraphExecDestroy(exec);
    cudaGraphDestroy(graph);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    release2();
    if (se != cudaSuccess) {
        cleanup();
        if (d_phase) cudaFree(d_phase);
        return fau_internal_fail(FAU_ERR_CUDA, cudaGetErrorString(se));
    }
    if (d_phase) {
        std::vector<unsigned long long> ph((size_t)kFastPhaseSlots * n);
        cudaMemcpy(ph.data(), d_phase, sizeof(unsigned long long) * ph.size(), cudaMemcpyDeviceToHost);
        cudaFree(d_phase);
        static const char* names_e[kPhaseSlots] = {"deferred_q", "ewald", "pairs", "reduce+B1", "decision", "commit",
                                                   "prepare", "B2(w0)", "compute(w1)", "B1(w1)", "B2(w1)",
                                                   "cutoff_pass(w1)", "pair_tasks(w1)", "prep:proposal",
                                                   "prep:positions", "prep:tables", "moves"};
        static const char* names_f[kFastPhaseSlots] = {
            "P:commit_data", "P:prepare", "P:copies", "P:B1", "P:decision", "P:commit", "P:B2",
            "C:preload", "C:ewald", "C:pairs", "C:sums", "C:B1", "C:decision", "C:q_update", "C:B2", "moves",
            "prep:scalar_rest", "prep:tables", "prep:entries", "C:pairs_pre", "prep:fp64_add", "P:proposal",
            "prep:to_fixed", "prep:cells"};
        for (int part = 0; part < 2; part++) {
            const int r0 = part == 0 ? 0 : nfast, r1 = part == 0 ? nfast : n;
            if (r1 <= r0) continue;
            const int ns = part == 0 ? kFastPhaseSlots : kPhaseSlots;
            const int mslot = part == 0 ? 15 : kPhaseSlots - 1;
            double tot[kFastPhaseSlots] = {0};
            for (int r = r0; r < r1; r++)
                for (int j = 0; j < ns; j++) tot[j] += (double)ph[(size_t)r * kFastPhaseSlots + j];
            const double mv = tot[mslot] > 0 ? tot[mslot] : 1.0;
            std::fprintf(stderr, "FAU_PHASE_TIMING %s cycles per move:", part == 0 ? "pipelined" : "chain");
            for (int j = 0; j < ns; j++)
                if (j != mslot && tot[j] > 0)
                    std::fprintf(stderr, " %s=%.0f", part == 0 ? names_f[j] : names_e[j], tot[j] / mv);
            std::fprintf(stderr, " (moves %.0f)\n", tot[mslot]);
        }
    }
    fau_batch_stats S{};
    int derr = FAU_OK;
    for (int i = 0; i < n; i++) {
        S.moves += (int64_t)(s1[i].moves - s0[i].moves);
        S.accepted += (int64_t)(s1[i].accepted - s0[i].accepted);
        S.pair_evals += (int64_t)(s1[i].pair_evals - s0[i].pair_evals);
        S.k_updates += (int64_t)(s1[i].k_updates - s0[i].k_updates);
        if (s1[i].err != FAU_OK && derr == FAU_OK) derr = s1[i].err;
        S.du_err_scaled_max = std::max(S.du_err_scaled_max, s1[i].audit_scaled);
        S.du_err_rel_max = std::max(S.du_err_rel_max, s1[i].audit_rel);
        S.du_err_samples += (int64_t)(s1[i].audit_samples - s0[i].audit_samples);
    }
    if (P->cycles_out)
        for (int i = 0; i < n; i++) P->cycles_out[i] = (uint64_t)(s1[i].cycles - s0[i].cycles);
    if (P->moves_out) // blocked launches run every block in full; otherwise the one launch's count
        for (int i = 0; i < n; i++)
            P->moves_out[i] = blocked ? (int64_t)(pt_lens ? nm[i] : blk_moves) * nblk : (int64_t)s1[i].consumed;
    S.swaps_attempted = (int64_t)pst[0];
    S.swaps_accepted = (int64_t)pst[1];
    S.device_ms = ms;
    if (stats) *stats = S;
    cleanup();
#undef BTRY
    if (derr != FAU_OK) {
        // clear the device error flags so the systems stay usable
        for (int i = 0; i < n; i++) cudaMemsetAsync(&dsys[i]->err, 0, sizeof(int), st);
        cudaStreamSynchronize(st);
        if (derr == FAU_ERR_CAPACITY) {
            // a chain filled a cell: its move is committed and its chain stopped after it; the
            // cells are regrown so that the caller can continue every system at counter + moves_out
            for (int i = 0; i < n; i++)
                if (s1[i].err == FAU_ERR_CAPACITY) {
                    const int e = fau_internal_sys_regrow(systems[i]);
                    if (e != FAU_OK) return e;
                }
            return fau_internal_fail(derr, "a cell list filled up: capacity doubled; continue the systems at "
                                           "counter + moves_out");
        }
        return fau_internal_fail(derr, "a system in the batch reported a device error");
    }
    return rc;
}

extern "C" int fau_run_proposals_batch(fau_ctx* ctx, fau_sys* const* systems, int n, const fau_proposal* props,
                                       const int64_t* offsets, uint8_t* acc_out, double* du_out,
                                       fau_batch_stats* stats)
{
    const NvtxRange nvtx_range("fau_run_proposals_batch");
    if (!ctx || !systems || !props || !offsets || n < 1)
        return fau_internal_fail(FAU_ERR_ARG, "invalid batch arguments");
    cudaStream_t st;
    int device;
    fau_internal_ctx_stream(ctx, &st, &device);
    if (cudaSetDevice(device) != cudaSuccess) return fau_internal_fail(FAU_ERR_CUDA, "cudaSetDevice failed");
    std::vector<DevSys*> dsys(n);
    std::vector<long long> nm(n), off(n);
    std::vector<int> Kv(n), ncv(n);
    std::vector<uint8_t> fast(n, 0);
    const long long total = offsets[n];
    if (offsets[0] != 0 || total < 0) return fau_internal_fail(FAU_ERR_ARG, "offsets must start at 0");
    for (int i = 0; i < n; i++) {
        fau_ctx* c2;
        int K, np, ng, mo, knc;
        double tr;
        fau_internal_sys_view(systems[i], &c2, &dsys[i], &K, &np, &ng, &mo, &tr, &knc);
        if (c2 != ctx) return fau_internal_fail(FAU_ERR_ARG, "system from another context");
        if (offsets[i + 1] < offsets[i]) return fau_internal_fail(FAU_ERR_ARG, "offsets not sorted");
        nm[i] = offsets[i + 1] - offsets[i];
        off[i] = offsets[i];
        Kv[i] = K;
        ncv[i] = knc;
        // systems of atomic groups only run in the pipelined kernel (single-atom moves), the others
        // in the 256-thread chain kernel; the kernels check every proposal as they read it
        fast[i] = fau_internal_sys_all_atomic(systems[i]) && knc <= kFastMaxNc && !fau_internal_sys_maxe(systems[i]);
    }
    // FP64 systems: the FP64 chain kernel (a batch holds FP64 systems only or none)
    const int f64 = fp64_batch(systems, n);
    if (f64 < 0) return f64 == -1 ? fau_internal_fail(FAU_ERR_ARG, kFp64Mixed) : fau_internal_fail(FAU_ERR_ARG, kFp64Form);
    const int g64 = f64 > 0 ? max_groups(systems, n) : 0;
    if (f64)
        for (int i = 0; i < n; i++) fast[i] = 0;
    // kernel order puts the pipelined-kernel systems first
    std::vector<int> order;
    order.reserve(n);
    for (int i = 0; i < n; i++)
        if (fast[i]) order.push_back(i);
    const int nfast = (int)order.size();
    for (int i = 0; i < n; i++)
        if (!fast[i]) order.push_back(i);
    const int nexact = n - nfast;
    int Kf = 0, ncf = 0, ntf = 1, Ke = 0, nce = 0;
    bool occf = false;
    for (int r = 0; r < n; r++) {
        const int i = order[r];
        if (r < nfast) {
            Kf = std::max(Kf, Kv[i]);
            ncf = std::max(ncf, ncv[i]);
            ntf = std::max(ntf, fau_internal_sys_classes(systems[i]));
            occf = occf || fau_internal_sys_occ(systems[i]);
        }
        else {
            Ke = std::max(Ke, Kv[i]);
            nce = std::max(nce, ncv[i]);
        }
    }
    if (f64 ? fp64_smem_bytes(Ke, g64) + 16384 > 227 * 1024
            : ((nexact && (Ke > chain_max_k(256) || chain_smem_bytes(Ke, nce) + 16384 > 227 * 1024)) ||
               (nfast && fast_smem_bytes_total(Kf, ncf, ntf) > 227 * 1024)))
        return fau_internal_fail(FAU_ERR_ARG, "too many k-vectors (FP64 chains: k-vectors and groups) for the chain kernel");
    if (f64 && prepare_fp64(Ke, g64, false) != cudaSuccess)
        return fau_internal_fail(FAU_ERR_CUDA, "FP64 chain kernel attributes");
    // systems of molecular groups only whose proposals are all molecular (or empty) run in the
    // pipelined molecular kernel when every other-than-single-atom system qualifies; otherwise
    // the chain kernel runs them (it takes every proposal kind)
    bool use_mol = !f64 && nexact > 0;
    if (const char* mk = std::getenv("FAU_MOL_KERNEL"); mk && mk[0] == '0') use_mol = false;
    for (int r = nfast; r < n && use_mol; r++) {
        const int i = order[r];
        fau_ctx* c2;
        int K, np, ng, mo, knc;
        double tr;
        DevSys* dd;
        fau_internal_sys_view(systems[i], &c2, &dd, &K, &np, &ng, &mo, &tr, &knc);
        if (!mo || fau_internal_sys_maxe(systems[i])) use_mol = false;
        for (long long m = off[i]; m < off[i] + nm[i] && use_mol; m++)
            if (props[m].kind != FAU_MOVE_MOLECULAR && props[m].kind != FAU_MOVE_NONE) use_mol = false;
    }
    if (use_mol && mol_smem_bytes_total(Ke, nce) + 24576 > 227 * 1024) use_mol = false;
    if (use_mol && mol_dispatch_256(ChainArgs{}, 0, Ke, nce, nullptr, true) != cudaSuccess)
        return fau_internal_fail(FAU_ERR_CUDA, "molecular kernel attributes");
    // proposals in pinned host memory that the device can address are read in place by the
    // pipelined kernel (streamed through its shared-memory ring while the chains run); otherwise
    // they are staged with one copy
    const fau_proposal* dprops = nullptr;
    if (nexact == 0) {
        cudaPointerAttributes pa{};
        if (cudaPointerGetAttributes(&pa, props) == cudaSuccess && pa.type == cudaMemoryTypeHost && pa.devicePointer)
            dprops = static_cast<const fau_proposal*>(pa.devicePointer);
        cudaGetLastError();
    }
    const long long staged = dprops ? 0 : total;
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    const size_t o_sys = 0, o_ksys = al(o_sys + 8 * n), o_nm = al(o_ksys + 8 * n), o_off = al(o_nm + 8 * n),
                 o_sum = al(o_off + 8 * n),
                 o_props = al(o_sum + sizeof(SysSummary) * n), o_acc = al(o_props + sizeof(fau_proposal) * staged),
                 o_du = al(o_acc + total), bytes = al(o_du + 8 * total);
    unsigned char* dbuf = nullptr;
    if (fau_internal_ctx_scratch(ctx, bytes, reinterpret_cast<void**>(&dbuf)) != FAU_OK)
        return fau_internal_fail(FAU_ERR_OOM, "batch staging allocation");
    auto done = [&](int code, const char* msg) { // dbuf is the context's scratch
        return code == FAU_OK ? FAU_OK : fau_internal_fail(code, msg);
    };
    DevSys* const* d_sys = reinterpret_cast<DevSys* const*>(dbuf + o_sys);
    SysSummary* d_sum = reinterpret_cast<SysSummary*>(dbuf + o_sum);
    std::vector<SysSummary> s0(n), s1(n);
    std::vector<DevSys*> ksys(n);
    std::vector<long long> knm(n), koff(n);
    for (int r = 0; r < n; r++) {
        ksys[r] = dsys[order[r]];
        knm[r] = nm[order[r]];
        koff[r] = off[order[r]];
    }
    if (cudaMemcpyAsync(dbuf + o_sys, dsys.data(), 8 * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dbuf + o_ksys, ksys.data(), 8 * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dbuf + o_nm, knm.data(), 8 * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(dbuf + o_off, koff.data(), 8 * n, cudaMemcpyHostToDevice, st) != cudaSuccess ||
        (staged && cudaMemcpyAsync(dbuf + o_props, props, sizeof(fau_proposal) * staged, cudaMemcpyHostToDevice,
                                   st) != cudaSuccess))
        return done(FAU_ERR_CUDA, "proposal upload failed");
    gather_kernel<<<(n + 127) / 128, 128, 0, st>>>(d_sys, n, d_sum);
    cudaMemcpyAsync(s0.data(), d_sum, sizeof(SysSummary) * n, cudaMemcpyDeviceToHost, st);
    ChainArgs a{};
    a.sys = reinterpret_cast<DevSys* const*>(dbuf + o_ksys);
    a.audit = 1;
    a.n_moves = reinterpret_cast<const long long*>(dbuf + o_nm);
    a.prop_off = reinterpret_cast<const long long*>(dbuf + o_off);
    a.props = dprops ? dprops : reinterpret_cast<const fau_proposal*>(dbuf + o_props);
    a.acc_out = acc_out ? reinterpret_cast<uint8_t*>(dbuf + o_acc) : nullptr;
    a.du_out = du_out ? reinterpret_cast<double*>(dbuf + o_du) : nullptr;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    ChainArgs ae = a;
    ae.sys = a.sys + nfast;
    ae.n_moves = a.n_moves + nfast;
    ae.prop_off = a.prop_off + nfast;
    cudaStream_t st2 = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    bool ok = true;
    if (nfast && nexact) {
        ok = cudaStreamCreateWithFlags(&st2, cudaStreamNonBlocking) == cudaSuccess &&
             cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming) == cudaSuccess;
    }
    cudaEventRecord(e0, st);
    if (ok && nexact) {
        if (nfast) {
            ok = cudaEventRecord(fork_ev, st) == cudaSuccess && cudaStreamWaitEvent(st2, fork_ev, 0) == cudaSuccess &&
                 (use_mol ? mol_dispatch_256(ae, nexact, Ke, nce, st2, false)
                          : launch_chain(ae, nexact, Ke, nce, 256, false, st2)) == cudaSuccess &&
                 launch_probe_audit(ae.sys, nexact, st2) == cudaSuccess &&
                 cudaEventRecord(join_ev, st2) == cudaSuccess;
        }
        else if (f64) {
            ok = launch_fp64(ae, nexact, Ke, g64, false, st) == cudaSuccess;
        }
        else {
            ok = (use_mol ? mol_dispatch_256(ae, nexact, Ke, nce, st, false)
                          : launch_chain(ae, nexact, Ke, nce, 256, false, st)) == cudaSuccess &&
                 launch_probe_audit(ae.sys, nexact, st) == cudaSuccess;
        }
    }
    if (ok && nfast) ok = launch_fast(a, nfast, Kf, ncf, ntf, 4, false, occf, st) == cudaSuccess;
    if (ok && nfast) ok = launch_fast_audit(a.sys, nfast, st) == cudaSuccess;
    if (ok && nfast && a.du_out) {
        unpack_du_kernel<<<nfast, 256, 0, st>>>(a.du_out, a.prop_off, a.n_moves);
        ok = cudaGetLastError() == cudaSuccess;
    }
    if (ok && nfast && nexact) ok = cudaStreamWaitEvent(st, join_ev, 0) == cudaSuccess;
    if (!ok) {
        cudaStreamSynchronize(st);
        if (st2) cudaStreamDestroy(st2);
        if (fork_ev) cudaEventDestroy(fork_ev);
        if (join_ev) cudaEventDestroy(join_ev);
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        return done(FAU_ERR_CUDA, "chain launch failed");
    }
    cudaEventRecord(e1, st);
    gather_kernel<<<(n + 127) / 128, 128, 0, st>>>(d_sys, n, d_sum);
    cudaMemcpyAsync(s1.data(), d_sum, sizeof(SysSummary) * n, cudaMemcpyDeviceToHost, st);
    if (acc_out) cudaMemcpyAsync(acc_out, dbuf + o_acc, total, cudaMemcpyDeviceToHost, st);
    if (du_out) cudaMemcpyAsync(du_out, dbuf + o_du, 8 * total, cudaMemcpyDeviceToHost, st);
    const cudaError_t se = cudaStreamSynchronize(st);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (st2) cudaStreamDestroy(st2);
    if (fork_ev) cudaEventDestroy(fork_ev);
    if (join_ev) cudaEventDestroy(join_ev);
    if (se != cudaSuccess) return done(FAU_ERR_CUDA, cudaGetErrorString(se));
    fau_batch_stats S{};
    int derr = FAU_OK;
    for (int i = 0; i < n; i++) {
        S.moves += (int64_t)(s1[i].moves - s0[i].moves);
        S.accepted += (int64_t)(s1[i].accepted - s0[i].accepted);
        S.pair_evals += (int64_t)(s1[i].pair_evals - s0[i].pair_evals);
        S.k_updates += (int64_t)(s1[i].k_updates - s0[i].k_updates);
        if (s1[i].err != FAU_OK && derr == FAU_OK) derr = s1[i].err;
        S.du_err_scaled_max = std::max(S.du_err_scaled_max, s1[i].audit_scaled);
        S.du_err_rel_max = std::max(S.du_err_rel_max, s1[i].audit_rel);
        S.du_err_samples += (int64_t)(s1[i].audit_samples - s0[i].audit_samples);
    }
    S.device_ms = ms;
    if (stats) *stats = S;
    if (derr != FAU_OK) {
        for (int i = 0; i < n; i++) cudaMemsetAsync(&dsys[i]->err, 0, sizeof(int), st);
        cudaStreamSynchronize(st);
        return done(derr, "a system in the batch reported a device error");
    }
    return done(FAU_OK, nullptr);
}

// ---------------------------------------------------------------- FP32 peak probe
namespace {
__global__ void fma_probe_kernel(float* out, int iters, float a, float b)
{
    float x0 = threadIdx.x * 1e-7f, x1 = x0 + 1.f, x2 = x0 + 2.f, x3 = x0 + 3.f;
    float x4 = x0 + 4.f, x5 = x0 + 5.f, x6 = x0 + 6.f, x7 = x0 + 7.f;
    for (int i = 0; i < iters; i++) {
#pragma unroll
        for (int j = 0; j < 16; j++) {
            x0 = fmaf(x0, a, b); x1 = fmaf(x1, a, b); x2 = fmaf(x2, a, b); x3 = fmaf(x3, a, b);
            x4 = fmaf(x4, a, b); x5 = fmaf(x5, a, b); x6 = fmaf(x6, a, b); x7 = fmaf(x7, a, b);
        }
    }
    const float s = ((x0 + x1) + (x2 + x3)) + ((x4 + x5) + (x6 + x7));
    if (s == 12345.678f) out[0] = s; // keeps the chains live
}
} // namespace

extern "C" int fau_measure_fp32_peak(fau_ctx* ctx, double* tflops)
{
    if (!ctx || !tflops) return fau_internal_fail(FAU_ERR_ARG, "null argument");
    cudaStream_t st;
    int device;
    fau_internal_ctx_stream(ctx, &st, &device);
    cudaSetDevice(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    float* d = nullptr;
    if (cudaMalloc(&d, sizeof(float)) != cudaSuccess) return fau_internal_fail(FAU_ERR_OOM, "probe allocation");
    const int blocks = sms * 8, threads = 256, iters = 4096;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    fma_probe_kernel<<<blocks, threads, 0, st>>>(d, 64, 0.999999f, 1e-7f); // warm up
    double best = 0.0;
    for (int r = 0; r < 5; r++) {
        cudaEventRecord(e0, st);
        fma_probe_kernel<<<blocks, threads, 0, st>>>(d, iters, 0.999999f, 1e-7f);
        cudaEventRecord(e1, st);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8 * 16 * (double)iters * blocks * threads;
        best = std::max(best, flops / (ms * 1e-3) / 1e12);
    }
    const cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    if (e != cudaSuccess) return fau_internal_fail(FAU_ERR_CUDA, cudaGetErrorString(e));
    *tflops = best;
    return FAU_OK;
}
