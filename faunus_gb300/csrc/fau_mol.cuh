// fau_mol.cuh -- pipelined chain kernel for molecular moves (TranslateRotate,
// src/move.cpp:1670-1689) of rigid molecules with device (Philox) proposals.
//
// One CTA runs one system's Markov chain.  The chain kernel prepares move t+1
// (FP64 translation + quaternion rotation of every atom, wrap, fixed-point
// records, phase tables) after the Metropolis decision of move t, on the
// critical path; measured on rigid water that preparation is a serial FP64 chain
// of ~20k cycles per move, as long as the whole pair phase.  Here warp 0 prepares
// move t+1 speculatively while warps 1..NW-1 evaluate move t (Ewald dQ and the
// GroupCutoff-compacted group-vs-rest pair sum), into a second MoveShared and a
// second set of phase tables.  After the decision and commit of move t, a
// prepared move that picked the same group is prepared again from the committed
// positions (the only state a molecular move's preparation reads that move t can
// change: the moved group's atoms and mass centre).  Everything else -- term
// order, precision, guard bands, the Q(k) bookkeeping and the FP64 decision --
// is the chain kernel's, so both kernels give the same chains for the same
// proposal stream, barring near ties (the compute warps sum in a different order).
#pragma once

#include "fau_chain.cuh"

namespace fau {

__device__ __forceinline__ void compute_barrier(int nthreads)
{
    asm volatile("bar.sync 1, %0;" ::"r"(nthreads) : "memory");
}

// One (neighbour group, moved atom) task for an NB-site neighbour: its NB records loaded
// together, the 2 NB pair distances formed, and -- unless one lies in a guard band, where
// pair_u32's FP64 check must decide (returns false) -- all pair energies evaluated at once,
// then accumulated in the per-pair order of the general path.
template <int NB>
__device__ __forceinline__ bool mol_task_fast(const DevSys& S, const PairF* pt, int nt, int ta, uint4 ra_n, uint4 ra_o,
                                              int hb, bool do_n, bool do_o, FF& acc, int& flags,
                                              unsigned long long& n_pairs)
{
    if (S.terms & FAU_PAIR_SPLINE) return false; // tabulated pairs: the general path
    uint4 rb[NB];
#pragma unroll
    for (int j = 0; j < NB; j++) rb[j] = S.rec[hb + j];
    PairF pp[2 * NB];
    float r2[2 * NB];
    bool near = false;
#pragma unroll
    for (int j = 0; j < NB; j++) {
        const PairF p = pt[ta * nt + (int)(rb[j].w >> 24)];
        pp[j] = p;
        pp[NB + j] = p;
        r2[j] = r2_fixed(S, ra_n, rb[j]);
        r2[NB + j] = r2_fixed(S, ra_o, rb[j]);
        near |= (do_n && pair_near(S, p, r2[j])) || (do_o && pair_near(S, p, r2[NB + j]));
    }
    if (near) return false;
    // the LJ/WCA part of pair j is skipped where it is exactly zero for every lane of the warp
    // (tasks are ordered by moved atom, so a warp mostly shares it: for SPC/E only O-O pairs remain)
    bool lj[2 * NB];
    const unsigned act = __activemask();
#pragma unroll
    for (int j = 0; j < NB; j++) {
        const float tiny = pp[j].s2 * 1e-6f;
        const bool need = !(pp[j].e4 == 0.f) || !(pp[j].s2 == pp[j].s2) || r2[j] < tiny || r2[NB + j] < tiny;
        lj[j] = lj[NB + j] = __any_sync(act, need) != 0;
    }
    float u[2 * NB];
    bool fi[2 * NB], fn[2 * NB];
    pair_far_multi<2 * NB>(S, pp, r2, u, fi, fn, lj);
#pragma unroll
    for (int j = 0; j < NB; j++) {
        add_pair(acc, flags, do_n ? u[j] : 0.f, do_o ? u[NB + j] : 0.f, do_n && fi[j], do_o && fi[NB + j],
                 do_n && fn[j], do_o && fn[NB + j]);
    }
    n_pairs += (unsigned long long)NB * ((do_n ? 1 : 0) + (do_o ? 1 : 0));
    return true;
}

// mass-centre cell of an FP64 mass centre: floor((x + L/2) / side), clamped to the grid
__device__ __forceinline__ int gcell_of(const DevSys& S, const double* x, int* c3)
{
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int v = (int)floor(__dmul_rn(__dadd_rn(x[d], S.half[d]), S.ginv[d]));
        c3[d] = min(max(v, 0), S.gdim[d] - 1);
    }
    return c3[0] + S.gdim[0] * (c3[1] + S.gdim[1] * c3[2]);
}

// The cells whose groups are GroupCutoff candidates of one molecular move: every cell within
// one of the moved group's old or new cell (a box of at most 4 x 4 x 4 for a move shorter than
// a cell); n = -1 for a longer move (every group is a candidate) or without cells.
template <bool B>
struct ByCell { // compile-time choice of the candidate enumeration (separate code for each)
    static constexpr bool value = B;
};

struct GBox {
    int n, c_old, c_new, pad;
    int cells[64];
};

__device__ __forceinline__ void gbox_prepare(const DevSys& S, const MoveShared& ms, GBox& b, int lane)
{
    if (S.gncell == 0 || ms.kind != FAU_MOVE_MOLECULAR || ms.stop) {
        if (lane == 0) b.n = -1;
        return;
    }
    int co[3], cn[3], start[3], span[3];
    const int c_old = gcell_of(S, S.g_cm + 3 * ms.index, co);
    const int c_new = gcell_of(S, ms.cm_new, cn);
#pragma unroll
    for (int d = 0; d < 3; d++) {
        const int G = S.gdim[d];
        int dd = cn[d] - co[d]; // minimum-image cell offset
        if (2 * dd > G) dd -= G;
        else if (2 * dd < -G) dd += G;
        const int lo = min(0, dd) - 1, hi = max(0, dd) + 1;
        span[d] = hi - lo + 1;
        start[d] = co[d] + lo;
        if (span[d] >= G) {
            span[d] = G;
            start[d] = 0;
        }
    }
    const int n = span[0] * span[1] * span[2];
    for (int e = lane; e < 64 && e < n; e += 32) {
        const int ex = e % span[0], ey = (e / span[0]) % span[1], ez = e / (span[0] * span[1]);
        int w[3] = {start[0] + ex, start[1] + ey, start[2] + ez};
#pragma unroll
        for (int d = 0; d < 3; d++) w[d] = (w[d] % S.gdim[d] + S.gdim[d]) % S.gdim[d];
        b.cells[e] = w[0] + S.gdim[0] * (w[1] + S.gdim[1] * w[2]);
    }
    if (lane == 0) {
        b.n = n <= 64 ? n : -1;
        b.c_old = c_old;
        b.c_new = c_new;
    }
}

// the kernel's static shared memory, declared once for both instances of its body
template <int NT>
struct __align__(16) MolShared {
    static constexpr int NW = NT / 32, NWC = NW - 1, CH = 6 * (NT - 32);
    DevSys Ssh;
    PairF pt[kMaxITypes * kMaxITypes];
    MoveShared msb[2];
    FF red_a[NW];
    int red_f[NW];
    uint32_t nbl[CH];   // neighbour group | interacting states
    uint32_t nbl_b[CH]; // its first particle | atom count << 24
    int nbl_wcnt[2][NWC]; // survivors per compute warp: single pass | current chunk
    int sh_prev_accept, sh_stop, sh_time_up, pad;
    GBox gbx[2];        // the candidate cells of moves mv (gbx[mv & 1]) and mv + 1
    unsigned long long sh_t0; // globaltimer at the start (time-budgeted launches)
    long long sh_consumed;
    unsigned long long red_u[NW][2];
};

// CELLS: the system has mass-centre cells (its GroupCutoff candidates come from them); the
// body is compiled for each case, so systems without cells run exactly the code they had.
// HOST: proposals from A.props (checked by prepare_move), accept flags and dU written to
// A.acc_out / A.du_out; otherwise the device RNG's proposals.
template <int NT, bool CELLS, bool HOST>
__device__ __forceinline__ void mol_chain_body(const ChainArgs& A, MolShared<NT>& sm)
{
    constexpr int NW = NT / 32;
    constexpr int NWC = NW - 1;   // compute warps
    constexpr int NTC = NT - 32;  // compute threads
    constexpr int RC = 6;         // candidate groups per compute thread per chunk (1344: one chunk
    constexpr int CH = RC * NTC;  // covers a 1,000-molecule system, one barrier pair per move)
    constexpr int SB = 2;         // candidates whose loads are in flight together (RC % SB == 0)
    constexpr int SEG = RC * 32;  // list slots of one compute warp (its candidates in one chunk)
    static_assert(CH == MolShared<NT>::CH, "list size");
    const long long t_start = clock64();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int ctid = tid - 32; // compute-thread index (warps 1..)
    DevSys& G = *A.sys[blockIdx.x];
    DevSys& Ssh = sm.Ssh;
    for (int w = tid; w < (int)(sizeof(DevSys) / 8); w += NT)
        reinterpret_cast<unsigned long long*>(&Ssh)[w] = reinterpret_cast<const unsigned long long*>(&G)[w];
    __syncthreads();
    const DevSys& S = Ssh;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int K = (S.flags & SYS_EWALD) ? S.K : 0;
    const int nc = S.knc;
    const int TS = 2 * nc + 1;
    float2* Qb = reinterpret_cast<float2*>(smem_raw);
    float2* pend = Qb + K;
    float2* dlt = pend + K;
    int* kidx = reinterpret_cast<int*>(dlt + K);
    float* Af = reinterpret_cast<float*>(kidx + K);
    float2* tabs = reinterpret_cast<float2*>(Af + K); // two sets of kTableAtoms * 6 * TS phase tables
    const int tab_len = kTableAtoms * 6 * TS;

    auto& pt = sm.pt;
    auto& msb = sm.msb;
    auto& red_a = sm.red_a;
    auto& red_f = sm.red_f;
    auto& nbl = sm.nbl;
    auto& nbl_b = sm.nbl_b;
    auto& nbl_wcnt = sm.nbl_wcnt;
    int& sh_prev_accept = sm.sh_prev_accept;
    int& sh_stop = sm.sh_stop;
    int& sh_time_up = sm.sh_time_up;
    auto& gbx = sm.gbx;
    unsigned long long& sh_t0 = sm.sh_t0;
    long long& sh_consumed = sm.sh_consumed;

    const float rec_pref_f = (float)S.rec_pref;
    for (int k = tid; k < K; k += NT) {
        const double2 q = S.Q[k];
        Qb[k] = make_float2((float)q.x, (float)q.y);
        pend[k] = S.qpend[k]; // where the previous launch left the pending changes
        dlt[k] = S.qdlt[k];
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        kidx[k] = (nx + nc) | ((ny + nc) << 8) | ((nz + nc) << 16);
        Af[k] = rec_pref_f * S.Ak[k];
    }
    for (int t = tid; t < S.nt * S.nt; t += NT) pt[t] = S.pair[t];

    const long long nmoves = A.n_moves ? A.n_moves[blockIdx.x] : A.moves;
    const uint32_t sys_id = A.sys_ids ? A.sys_ids[blockIdx.x] : blockIdx.x;
    const unsigned long long ctr0 = A.counters ? A.counters[blockIdx.x] + A.counter_base : A.counter_base;
    const float dp_f = (float)(A.dp_sys ? A.dp_sys[blockIdx.x] : A.dp);
    const double dprot = A.dprot_sys ? A.dprot_sys[blockIdx.x] : A.dprot;
    const long long poff = A.prop_off ? A.prop_off[blockIdx.x] : 0;
    // the audit probe: one more move (the chain's next proposal; a host stream's last one again)
    // evaluated after the last one on the final state, never decided or committed; its FP32
    // energy change and the move go to the system's audit record for probe_audit_kernel
    const long long nloop = nmoves + (A.audit && nmoves > 0 && G.audit_rec ? 1 : 0);
    // move idx's proposal: the host's (A.props, checked by prepare_move) or the device RNG's
    auto proposal = [&](long long idx) -> Proposal {
        if constexpr (HOST) return load_proposal(A.props[poff + (idx < nmoves ? idx : nmoves - 1)]);
        else return philox_proposal(S, ctr0 + (unsigned long long)idx, sys_id, A.seed, dp_f, dprot, true);
    };
    const int nt = S.nt;

    unsigned long long n_acc = 0, n_pairs = 0, n_k = 0, n_mv = 0;
    int since_flush = S.q_since; // counted by the compute threads
    double energy = sys_energy(S), sum_du = 0.0; // the pipelined kernel's unfolded part folded in
    double M[3] = {S.M[0], S.M[1], S.M[2]};
    long long consumed = nmoves;
    bool counted = false; // the pair and k-vector counts were reduced before the audit probe
    int err_code = 0; // the status that ended the chain early (FAU_ERR_*), 0 if none

    // phase timers (profiling only): warp 0 (tid 0): 6 prepare ahead, 3 wait B1, 4 decision,
    // 5 commit (+ re-prepare), 7 B2; warp 1 (tid 32): 0 deferred Q, 1 Ewald, 11 GroupCutoff passes,
    // 12 pair tasks, 2 the rest of the pairs, 9 B1, 10 B2; last: moves
    const bool timing = A.phase_cycles != nullptr && (tid == 0 || tid == 32);
    unsigned long long tacc[kPhaseSlots] = {0};
    long long tprev = timing ? clock64() : 0;
    auto tick = [&](int slot) {
        if (timing) {
            const long long t = clock64();
            tacc[slot] += (unsigned long long)(t - tprev);
            tprev = t;
        }
    };
    if (tid == 0) {
        sh_prev_accept = S.q_valid; // the previous launch's last accepted change, if not yet folded
        sh_stop = 0;
        sh_time_up = 0;
        sh_t0 = global_ns();
    }
    if constexpr (CELLS) {
        // list the molecular groups by mass-centre cell, ascending within each cell (the lists
        // depend only on the mass centres: a chain split into launches sees the same ones)
        for (int c = tid; c < S.gncell; c += NT) S.gc_cnt[c] = 0;
        __syncthreads();
        for (int h = tid; h < S.n_groups; h += NT) {
            if (S.g_flags[h] & FAU_GROUP_ATOMIC) continue;
            int c3[3];
            const int c = gcell_of(S, S.g_cm + 3 * h, c3);
            const int slot = atomicAdd(&S.gc_cnt[c], 1);
            if (slot < S.gcap) S.gc_list[(size_t)c * S.gcap + slot] = h;
        }
        __syncthreads();
        for (int c = tid; c < S.gncell; c += NT) {
            const int n = S.gc_cnt[c];
            if (n > S.gcap) {
                sh_stop = FAU_ERR_CAPACITY; // no move runs: the caller sees the capacity error
                sh_consumed = 0;
                continue;
            }
            int* l = S.gc_list + (size_t)c * S.gcap;
            for (int i = 1; i < n; i++) { // insertion sort of a few dozen indices
                const int v = l[i];
                int j = i - 1;
                while (j >= 0 && l[j] > v) {
                    l[j + 1] = l[j];
                    j--;
                }
                l[j + 1] = v;
            }
        }
    }
    __syncthreads();
    if (warp == 0 && nmoves > 0) {
        const Proposal p = proposal(0);
        prepare_move(S, msb[0], p, lane, K ? tabs : nullptr, nc);
        if constexpr (CELLS) {
            __syncwarp();
            gbox_prepare(S, msb[0], gbx[0], lane);
        }
    }
    __syncthreads();

    for (long long mv = 0; mv < nloop; mv++) {
        const int cur = (int)(mv & 1);
        MoveShared& ms = msb[cur];
        MoveShared& mn = msb[cur ^ 1];
        const float2* tab = tabs + cur * tab_len;
        float2* tab_next = tabs + (cur ^ 1) * tab_len;
        const bool probe = mv == nmoves;
        if (sh_stop || (ms.stop && !probe) || (sh_time_up && !probe)) { // a NaN energy change ended the chain, a
            consumed = sh_stop ? sh_consumed : mv;          // proposal was invalid, or the time
            err_code = sh_stop ? sh_stop : ms.stop;         // budget is spent
            break;
        }
        if (probe && ms.stop) break; // no probe of an invalid proposal
        if (probe) { // the counts end before the probe's pair and k-vector evaluations
            unsigned long long a = n_pairs, b = n_k;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                a += __shfl_xor_sync(0xffffffffu, a, o);
                b += __shfl_xor_sync(0xffffffffu, b, o);
            }
            if (lane == 0) {
                sm.red_u[warp][0] = a;
                sm.red_u[warp][1] = b;
            }
            counted = true;
        }
        const int kind = ms.kind;
        const int m = ms.m;
        FF accp{0.f, 0.f}, accr{0.f, 0.f};
        int flags = 0;
        if (warp == 0) {
            // ---- speculative preparation of move mv+1 (reads only the group it moves)
            if (mv + 1 < nloop) {
                const Proposal p = proposal(mv + 1);
                tick(13);
                prepare_move(S, mn, p, lane, K ? tab_next : nullptr, nc, timing ? &tacc[14] : nullptr);
                if constexpr (CELLS) {
                    __syncwarp();
                    gbox_prepare(S, mn, gbx[cur ^ 1], lane);
                }
            }
            tick(6);
        }
        else {
            // ---- the previous move's Q(k) change (same k partition as the Ewald loop below)
            if (sh_prev_accept) {
                for (int k = ctid; k < K; k += NTC) {
                    float2 pe = pend[k];
                    const float2 d = dlt[k];
                    pe.x += d.x;
                    pe.y += d.y;
                    pend[k] = pe;
                }
                if (++since_flush == kFlushAccepts) {
                    since_flush = 0;
                    for (int k = ctid; k < K; k += NTC) {
                        double2 q = S.Q[k];
                        const float2 pe = pend[k];
                        q.x += (double)pe.x;
                        q.y += (double)pe.y;
                        S.Q[k] = q;
                        Qb[k] = make_float2((float)q.x, (float)q.y);
                        pend[k] = make_float2(0.f, 0.f);
                    }
                }
            }
            if (timing) {
                tick(0);
                if (tid == 32) tacc[kPhaseSlots - 1]++;
            }
            if (kind != FAU_MOVE_NONE) {
                if (K) {
                    const bool tables = m <= kTableAtoms;
                    for (int k = ctid; k < K; k += NTC) {
                        const int ki = kidx[k];
                        const int ix = ki & 0xff, iy = (ki >> 8) & 0xff, iz = ki >> 16;
                        float2 d = make_float2(0.f, 0.f);
                        for (int a = 0; a < m; a++) {
                            float2 eo, h;
                            if (tables) {
                                const float2* t = tab + a * 6 * TS;
                                eo = cmul(t[ix], cmul(t[TS + iy], t[2 * TS + iz]));
                                h = cmul(t[3 * TS + ix], cmul(t[4 * TS + iy], t[5 * TS + iz]));
                            }
                            else {
                                const int nx = ix - nc, ny = iy - nc, nz = iz - nc;
                                eo = eikr32(nx, ny, nz, ms.rec_old[a]);
                                const float3 g = ms.g[a];
                                float sh, ch;
                                sincospif(fmaf((float)nx, g.x, fmaf((float)ny, g.y, (float)nz * g.z)), &sh, &ch);
                                h = make_float2(ch, sh);
                            }
                            const float2 pp = cmul(eo, h);
                            const float f = 2.f * ms.q[a] * h.y;
                            d.x = fmaf(-f, pp.y, d.x);
                            d.y = fmaf(f, pp.x, d.y);
                        }
                        dlt[k] = d;
                        const float2 qb = Qb[k], pe = pend[k];
                        const float qx = qb.x + pe.x, qy = qb.y + pe.y;
                        const float cross = 2.f * fmaf(qx, d.x, qy * d.y);
                        const float dd = fmaf(d.x, d.x, d.y * d.y);
                        ff_add(accr, Af[k] * (cross + dd));
                    }
                    n_k += (unsigned long long)m * (unsigned long long)((K - ctid + NTC - 1) / NTC > 0
                                                                            ? (K - ctid + NTC - 1) / NTC
                                                                            : 0);
                }
                tick(1);
                // ---- group2all(group) with GroupCutoff
                const int g = ms.index;
                const uint4 cmo = ms.cmrec_old, cmn = ms.cmrec_new;
                const double cmo_d[3] = {S.g_cm[3 * g], S.g_cm[3 * g + 1], S.g_cm[3 * g + 2]};
                const int GN = S.n_groups;
                const int mol_g = S.n_mol > 0 ? S.g_molid[g] : 0;
                // The candidates: every group, or (mass-centre cells) the groups listed in the
                // move's candidate cells, in rounds of 32 slots of one cell.  Each warp holds the
                // cells' counts and the first round of each (lanes e and e + 32 for cell e).
                const GBox& gb = gbx[cur];
                const bool by_cell = CELLS && gb.n > 0;
                struct CellRounds {
                    int cnt_lo, cnt_hi, ex_lo, ex_hi, rounds;
                };
                auto cell_rounds = [&]() {
                    CellRounds c{0, 0, 0, 0, 0};
                    if (lane < gb.n) c.cnt_lo = min(S.gc_cnt[gb.cells[lane]], S.gcap);
                    if (lane + 32 < gb.n) c.cnt_hi = min(S.gc_cnt[gb.cells[lane + 32]], S.gcap);
                    const int r_lo = (c.cnt_lo + 31) >> 5, r_hi = (c.cnt_hi + 31) >> 5;
                    int in_lo = r_lo, in_hi = r_hi;
#pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const int a = __shfl_up_sync(0xffffffffu, in_lo, o), b = __shfl_up_sync(0xffffffffu, in_hi, o);
                        if (lane >= o) {
                            in_lo += a;
                            in_hi += b;
                        }
                    }
                    in_hi += __shfl_sync(0xffffffffu, in_lo, 31);
                    c.ex_lo = in_lo - r_lo;
                    c.ex_hi = in_hi - r_hi;
                    c.rounds = __shfl_sync(0xffffffffu, in_hi, 31);
                    return c;
                };
                // candidate q (q >> 5 is the same in a whole warp): its group, or -1
                auto cand = [&](auto cells, const CellRounds& c, int q) -> int {
                    if constexpr (!decltype(cells)::value) {
                        return q < GN ? q : -1;
                    }
                    else {
                        const int u = q >> 5;
                        if (u >= c.rounds) return -1;
                        const int e = __popc(__ballot_sync(0xffffffffu, lane < gb.n && c.ex_lo <= u)) +
                                      __popc(__ballot_sync(0xffffffffu, lane + 32 < gb.n && c.ex_hi <= u)) - 1;
                        int first, cnt;
                        if (e < 32) {
                            first = __shfl_sync(0xffffffffu, c.ex_lo, e);
                            cnt = __shfl_sync(0xffffffffu, c.cnt_lo, e);
                        }
                        else {
                            first = __shfl_sync(0xffffffffu, c.ex_hi, e - 32);
                            cnt = __shfl_sync(0xffffffffu, c.cnt_hi, e - 32);
                        }
                        const int slot = ((u - first) << 5) + lane;
                        return slot < cnt ? S.gc_list[(size_t)gb.cells[e] * S.gcap + slot] : -1;
                    }
                };
                // GroupCutoff tests of SB candidates per thread starting at `base`; the survivors
                // are counted in the warp's wc and listed in the warp's own segment (nbl_slot),
                // up to SEG of them, with the states they interact in and their particle extents
                auto compact = [&](auto cells, const CellRounds& c, int base, int& wc) {
                    int hh[SB], gfl[SB], gml[SB], gb0[SB], gb1[SB];
                    uint4 gcr[SB];
#pragma unroll
                    for (int r = 0; r < SB; r++) hh[r] = cand(cells, c, base + r * NTC + ctid);
#pragma unroll
                    for (int r = 0; r < SB; r++) { // all loads first: their latencies overlap
                        const int h = hh[r];
                        gfl[r] = h >= 0 ? S.g_flags[h] : FAU_GROUP_ATOMIC;
                        gcr[r] = h >= 0 ? S.g_cmrec[h] : make_uint4(0, 0, 0, 0);
                        gml[r] = (h >= 0 && S.n_mol > 0) ? S.g_molid[h] : 0;
                        gb0[r] = h >= 0 ? S.g_begin[h] : 0;
                        gb1[r] = h >= 0 ? S.g_begin[h + 1] : 0;
                    }
#pragma unroll
                    for (int r = 0; r < SB; r++) {
                        const int h = hh[r];
                        uint32_t e = 0;
                        if (h >= 0 && h != g && !(gfl[r] & FAU_GROUP_ATOMIC)) {
                            double c2 = S.cut_g2g2;
                            float c2f = S.cut_g2g2f;
                            if (S.n_mol > 0) {
                                const int kk = mol_g * S.n_mol + gml[r];
                                c2 = S.cut2_mol[kk];
                                c2f = S.cut2_molf[kk];
                            }
                            const bool cut_o = group_cut_rec(S, cmo, cmo_d, gcr[r], h, c2, c2f);
                            const bool cut_n = group_cut_rec(S, cmn, ms.cm_new, gcr[r], h, c2, c2f);
                            e = (cut_n ? 0u : kNblNew) | (cut_o ? 0u : kNblOld);
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, e != 0);
                        const int slot = wc + __popc(bal & ((1u << lane) - 1u));
                        if (e && slot < SEG) {
                            nbl[(warp - 1) * SEG + slot] = (uint32_t)h | e;
                            nbl_b[(warp - 1) * SEG + slot] = (uint32_t)gb0[r] | ((uint32_t)(gb1[r] - gb0[r]) << 24);
                        }
                        wc += __popc(bal);
                    }
                };
                // the compute warps' survivor counts (after a barrier); over: a segment overflowed
                auto read_counts = [&](const int* src, int (&wcl)[NWC], bool& over) {
                    int cnt = 0;
                    over = false;
#pragma unroll
                    for (int v = 0; v < NWC; v++) {
                        wcl[v] = src[v];
                        cnt += wcl[v];
                        over |= wcl[v] > SEG;
                    }
                    return cnt;
                };
                // one (neighbour group, moved atom) task per thread over the cnt listed groups
                auto pair_tasks = [&](const int (&wcl)[NWC], int cnt) {
                    for (int task = ctid; task < cnt * m; task += NTC) {
                        const int a = task / cnt, q = task - a * cnt; // moved-atom major
                        const int sl = nbl_slot(q, wcl, SEG);
                        const uint32_t ent = nbl[sl];
                        const bool do_n = (ent & kNblNew) != 0, do_o = (ent & kNblOld) != 0;
                        const uint32_t hbn = nbl_b[sl];
                        const int hb = (int)(hbn & 0xFFFFFFu), nb = (int)(hbn >> 24), he = hb + nb;
                        const uint4 ra_n = ms.rec_new[a], ra_o = ms.rec_old[a];
                        const int ta = ra_n.w >> 24;
                        // 3- and 4-site neighbours away from every guard band: all pairs of both
                        // states evaluated together (pair_far_multi)
                        bool done = false;
                        if (nb == 3) done = mol_task_fast<3>(S, pt, nt, ta, ra_n, ra_o, hb, do_n, do_o, accp, flags, n_pairs);
                        else if (nb == 4) done = mol_task_fast<4>(S, pt, nt, ta, ra_n, ra_o, hb, do_n, do_o, accp, flags, n_pairs);
                        if (done) continue;
                        for (int b = hb; b < he; b++) {
                            const uint4 rb = S.rec[b];
                            const int pidx = ta * nt + (int)(rb.w >> 24);
                            const PairF p = pt[pidx];
                            float uu[2] = {0.f, 0.f};
                            bool fi[2] = {false, false}, fn[2] = {false, false};
                            float mg = 0.f;
                            for (int st = 0; st < 2; st++) {
                                if (!(st ? do_o : do_n)) continue;
                                uu[st] = pair_u32(S, p, pidx, r2_fixed(S, st ? ra_o : ra_n, rb),
                                                  st ? ms.xo[a] : ms.xn[a], b, fi[st], fn[st], mg);
                                n_pairs++;
                            }
                            add_pair(accp, flags, uu[0], uu[1], fi[0], fi[1], fn[0], fn[1]);
                        }
                    }
                };
                // one pass over every candidate group: a single barrier pair per move while each
                // warp's survivors fit its segment (GroupCutoff keeps ~140 of any number of waters)
                int wl[NWC];
                bool over;
                {
                    int wc = 0;
                    if (by_cell) {
                        const CellRounds c = cell_rounds();
                        for (int base = 0; base < c.rounds * 32; base += SB * NTC) compact(ByCell<true>{}, c, base, wc);
                    }
                    else {
                        const CellRounds c{0, 0, 0, 0, 0};
                        for (int base = 0; base < GN; base += SB * NTC) compact(ByCell<false>{}, c, base, wc);
                    }
                    if (lane == 0) nbl_wcnt[0][warp - 1] = wc;
                }
                compute_barrier(NTC);
                tick(11);
                const int total = read_counts(nbl_wcnt[0], wl, over);
                if (!over) {
                    pair_tasks(wl, total);
                    compute_barrier(NTC);
                    tick(12);
                }
                else { // more survivors than a segment holds (long or no cutoff): chunks of CH
                       // candidates, SEG of them per warp (the single-pass counts stay untouched:
                       // every warp has read them to take this branch)
                    const CellRounds c = by_cell ? cell_rounds() : CellRounds{0, 0, 0, 0, 0};
                    const int n_cand = by_cell ? c.rounds * 32 : GN;
                    for (int base = 0; base < n_cand; base += CH) {
                        int wc = 0;
                        for (int r0 = 0; r0 < RC; r0 += SB) {
                            if (base + r0 * NTC >= n_cand) break; // uniform: the ballots stay full-warp
                            if (by_cell) compact(ByCell<true>{}, c, base + r0 * NTC, wc);
                            else compact(ByCell<false>{}, c, base + r0 * NTC, wc);
                        }
                        if (lane == 0) nbl_wcnt[1][warp - 1] = wc;
                        compute_barrier(NTC);
                        tick(11);
                        const int cnt = read_counts(nbl_wcnt[1], wl, over);
                        pair_tasks(wl, cnt);
                        compute_barrier(NTC);
                        tick(12);
                    }
                }
                for (int t = ctid; t < S.n_atomic; t += NTC) { // atomic groups are never cut
                    const int b = S.atomic_idx[t];
                    const uint4 rb = S.rec[b];
                    const int tb = rb.w >> 24;
                    for (int a = 0; a < m; a++) {
                        const int pidx = (ms.rec_new[a].w >> 24) * nt + tb;
                        const PairF p = pt[pidx];
                        float uu[2];
                        bool fi[2], fn[2];
                        float mg = 0.f;
                        for (int st = 0; st < 2; st++) {
                            fi[st] = false;
                            fn[st] = false;
                            uu[st] = pair_u32(S, p, pidx, r2_fixed(S, st ? ms.rec_old[a] : ms.rec_new[a], rb),
                                              st ? ms.xo[a] : ms.xn[a], b, fi[st], fn[st], mg);
                        }
                        add_pair(accp, flags, uu[0], uu[1], fi[0], fi[1], fn[0], fn[1]);
                        n_pairs += 2;
                    }
                }
            }
            tick(2);
            accp = ff_sum(accp, accr);
            float sc = 0.f;
            warp_reduce(accp, accr, sc, flags, false);
            if (lane == 0) {
                red_a[warp] = accp;
                red_f[warp] = flags;
            }
        }
        __syncthreads(); // B1
        tick(tid == 0 ? 3 : 9);
        if (warp == 0) {
            accp = (lane >= 1 && lane <= NWC) ? red_a[lane] : FF{0.f, 0.f};
            flags = (lane >= 1 && lane <= NWC) ? red_f[lane] : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                FF ta{__shfl_xor_sync(0xffffffffu, accp.hi, o), __shfl_xor_sync(0xffffffffu, accp.lo, o)};
                accp = ff_sum(accp, ta);
                flags |= __shfl_xor_sync(0xffffffffu, flags, o);
            }
            int accept = 0, stop = 0, cell_full = 0;
            double du_out = 0.0;
            if (lane == 0 && kind != FAU_MOVE_NONE) {
                double du_surf = 0.0;
                if (S.flags & SYS_SURFACE) {
                    double m2o = 0.0, m2n = 0.0;
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        const double mnv = __dadd_rn(M[d], ms.dM[d]);
                        m2o = __dadd_rn(m2o, __dmul_rn(M[d], M[d]));
                        m2n = __dadd_rn(m2n, __dmul_rn(mnv, mnv));
                    }
                    du_surf = S.surf_pref * (m2n - m2o);
                }
                const double fin = ff_value(accp) + (0.0 + du_surf);
                if (probe) { // the audit probe: recorded for probe_audit_kernel, not decided
                    ProbeRecord& pr = *reinterpret_cast<ProbeRecord*>(G.audit_rec);
                    pr.kind = kind;
                    pr.index = ms.index;
                    pr.m = m;
                    pr.first = ms.first;
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        pr.cm_new[d] = ms.cm_new[d];
                        pr.dM[d] = ms.dM[d];
                    }
                    pr.du_surf = du_surf;
                    G.audit_du = fin;
                    G.audit_pending = flags == 0 ? 1 : 0; // finite in both states
                }
                else {
                    const double du =
                        energy_change(fin, flags & F_NEW_INF, flags & F_OLD_INF, flags & F_NEW_NAN, flags & F_OLD_NAN);
                    const double x = du * S.beta_scale;
                    du_out = du;
                    if (isnan(x)) stop = FAU_ERR_NAN;
                    else accept = metropolis(x, ms.u) ? 1 : 0;
                    if (accept) {
                        n_acc++;
                        sum_du += du;
                        energy += du;
#pragma unroll
                        for (int d = 0; d < 3; d++) M[d] = __dadd_rn(M[d], ms.dM[d]);
                    }
                    if (!stop) n_mv++;
                }
            }
            if (probe && kind != FAU_MOVE_NONE && lane < m) {
                ProbeRecord& pr = *reinterpret_cast<ProbeRecord*>(G.audit_rec);
#pragma unroll
                for (int d = 0; d < 3; d++) pr.xn[lane][d] = ms.xn[lane][d];
            }
            // the probe neither decides nor commits: accept stays 0, so the pass's fold of the last
            // accepted change is the last (q_valid 0) and the loop ends after it
            if constexpr (HOST) {
                if (lane == 0 && !probe) { // per-move outputs of host-proposal batches
                    if (A.acc_out) A.acc_out[poff + mv] = (uint8_t)accept;
                    if (A.du_out) A.du_out[poff + mv] = du_out;
                }
            }
            accept = __shfl_sync(0xffffffffu, accept, 0);
            stop = __shfl_sync(0xffffffffu, stop, 0);
            tick(4);
            if (!stop && accept) {
                // ---- commit (State::sync trial -> accepted): positions, records, mass centre
                if (lane < m) {
                    const int i = ms.first + lane;
                    S.x[i] = ms.xn[lane][0];
                    S.y[i] = ms.xn[lane][1];
                    S.z[i] = ms.xn[lane][2];
                    S.rec[i] = ms.rec_new[lane];
                }
                if (lane == 0 && kind == FAU_MOVE_MOLECULAR) {
                    const int g = ms.index;
#pragma unroll
                    for (int d = 0; d < 3; d++) S.g_cm[3 * g + d] = ms.cm_new[d];
                    S.g_cmrec[g] = ms.cmrec_new;
                    const GBox& gb = gbx[cur];
                    if (CELLS && gb.c_old != gb.c_new) { // the group changes mass-centre cell
                        int* lo = S.gc_list + (size_t)gb.c_old * S.gcap;
                        const int no = min(S.gc_cnt[gb.c_old], S.gcap);
                        int i = 0;
                        while (i < no && lo[i] != g) i++;
                        for (; i + 1 < no; i++) lo[i] = lo[i + 1];
                        S.gc_cnt[gb.c_old] = no - 1;
                        int* ln = S.gc_list + (size_t)gb.c_new * S.gcap;
                        const int nn = S.gc_cnt[gb.c_new];
                        if (nn >= S.gcap) {
                            cell_full = 1; // listed nowhere until the next launch lists every group again
                        }
                        else {
                            int j = nn;
                            while (j > 0 && ln[j - 1] > g) {
                                ln[j] = ln[j - 1];
                                j--;
                            }
                            ln[j] = g;
                            S.gc_cnt[gb.c_new] = nn + 1;
                        }
                    }
                }
                __syncwarp();
                __threadfence_block();
                // the prepared next move read this group's old positions: prepare it again
                if (mv + 1 < nloop && mn.kind == FAU_MOVE_MOLECULAR && kind == FAU_MOVE_MOLECULAR &&
                    mn.index == ms.index) {
                    const Proposal p = proposal(mv + 1);
                    prepare_move(S, mn, p, lane, K ? tab_next : nullptr, nc);
                    if constexpr (CELLS) {
                        __syncwarp();
                        gbox_prepare(S, mn, gbx[cur ^ 1], lane);
                    }
                }
            }
            if (lane == 0) {
                sh_prev_accept = stop ? 0 : accept;
                if (stop) {
                    sh_stop = stop;
                    sh_consumed = mv;
                }
                else if (cell_full) { // this move is committed; the chain ends after it
                    sh_stop = FAU_ERR_CAPACITY;
                    sh_consumed = mv + 1;
                }
                if (A.time_budget_ns && global_ns() - sh_t0 >= A.time_budget_ns) sh_time_up = 1;
            }
            __syncwarp();
            tick(5);
        }
        __syncthreads(); // B2
        tick(tid == 0 ? 7 : 10);
    }
    if (timing)
        for (int j = 0; j < kPhaseSlots; j++)
            if (tacc[j]) atomicAdd(&A.phase_cycles[blockIdx.x * kFastPhaseSlots + j], tacc[j]);

    // the pending changes stay pending: the next launch continues from them exactly as the next
    // move would (the host folds them into the master before it reads Q)
    __syncthreads();
    for (int k = tid; k < K; k += NT) {
        S.qpend[k] = pend[k];
        S.qdlt[k] = dlt[k];
    }
    if (tid == 32) G.q_since = K ? since_flush : 0;
    auto& red_u = sm.red_u;
    if (!counted) {
        unsigned long long a = n_pairs, b = n_k;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_xor_sync(0xffffffffu, a, o);
            b += __shfl_xor_sync(0xffffffffu, b, o);
        }
        if (lane == 0) {
            red_u[warp][0] = a;
            red_u[warp][1] = b;
        }
    }
    __syncthreads();
    if (tid == 0) {
        unsigned long long pa = 0, kb = 0;
        for (int w = 0; w < NW; w++) {
            pa += red_u[w][0];
            kb += red_u[w][1];
        }
        G.pair_evals += pa;
        G.k_updates += kb;
        G.moves += n_mv;
        G.accepted += n_acc;
        G.sum_du += sum_du;
        G.energy = energy;
        G.e_acc_hi = G.e_acc_lo = 0.f;
#pragma unroll
        for (int d = 0; d < 3; d++) G.M[d] = M[d];
        // a stop in the last move ends the loop without passing its top
        if (!err_code && sh_stop) {
            err_code = sh_stop;
            consumed = sh_consumed;
        }
        if (err_code) G.err = err_code;
        G.consumed = consumed;
        G.q_valid = K ? sh_prev_accept : 0;
        G.cycles += (unsigned long long)(clock64() - t_start);
    }
}

template <int NT, int MINB, bool HOST>
__global__ void __launch_bounds__(NT, MINB) mol_chain_kernel(ChainArgs A)
{
    __shared__ MolShared<NT> sm;
    if (A.sys[blockIdx.x]->gncell > 0) mol_chain_body<NT, true, HOST>(A, sm);
    else mol_chain_body<NT, false, HOST>(A, sm);
}

// dynamic shared memory of the molecular kernel: the chain kernel's plus a second set of tables
__host__ __device__ inline size_t mol_smem_bytes(int K, int nc)
{
    return chain_smem_bytes_v2(K, nc) + (size_t)kTableAtoms * 6 * (2 * nc + 1) * sizeof(float2);
}

template <int NT, int MINB, bool HOST>
cudaError_t launch_mol_inst(const ChainArgs& a, int nblocks, int K, int nc, cudaStream_t st, bool prepare_only)
{
    static size_t granted = 0;
    const size_t smem = mol_smem_bytes(K, nc);
    if (smem > granted || granted == 0) {
        cudaError_t e = cudaFuncSetAttribute(mol_chain_kernel<NT, MINB, HOST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        granted = smem;
    }
    if (prepare_only) return cudaSuccess;
    mol_chain_kernel<NT, MINB, HOST><<<nblocks, NT, smem, st>>>(a);
    return cudaGetLastError();
}

} // namespace fau
