// fau_fp64.cu -- FP64 replica chains: the persistent Metropolis chain in plain FP64 arithmetic,
// one CTA per system, for systems made with FAU_PREC_FP64.
//
// The arithmetic of the plain single-system FP64 form (plain_pair_kernel, plain_ewald_kernel and
// the host decision of fau_trial_atomic / fau_trial_group) run as a batched chain: the move, its
// energy change, the Metropolis decision and the commit stay on the device, so a batch of FP64
// systems runs as a persistent launch instead of one host round trip a move.  One loop
// iteration is one MetropolisMonteCarlo::performMove (src/montecarlo.cpp:139-187) of
// AtomicTranslateRotate (src/move.cpp:225-293) or TranslateRotate (src/move.cpp:1670-1689):
//
//   warp 0       the proposal (device Philox stream or the caller's proposals) and the trial
//                positions: prepare_move, the chain kernel's IEEE FP64 translation, rotation
//                about the new mass centre and wrapping, with fixed-point records
//   all threads  molecular moves: the GroupCutoff decision of every other group in both states
//                (mass-centre distances, src/energy.h:761-768)
//   all threads  the pair energy of the moved atoms in both states (Nonbonded group2all +
//                groupInternal, src/energy.h:886-914,1156-1195) against every other particle,
//                or for a single atom with a cell list against the particles of each state's
//                3x3x3 stencil (pair_u64 is exactly 0 beyond the pair cutoff, so both sums hold
//                the same terms), FP64 pair_u64 on FP64 minimum-image distances; the
//                reciprocal-space change d_k = sum_a q_a (e^{i k.r_new} - e^{i k.r_old}) from
//                FP64 phases and A_k (|Q_k + d_k|^2 - |Q_k|^2) (src/energy.cpp:219-247,524-531)
//   thread 0     the surface-term change (src/energy.cpp:466-482), getEnergyChange and
//                metropolisCriterion (src/montecarlo.cpp:17-34,193-209) on the FP64 sum, and
//                on accept the commit (positions, records, cell list or mass centre)
//   all threads  Q_k += d_k on accept (Ewald::sync, src/energy.cpp:640-658)
//
// Every sum is FP64 in a fixed order (per thread, then a shuffle tree, then the warps in index
// order), so a chain's result depends only on its system, proposals and seed.
#include "fau_chain.cuh"

namespace fau {
namespace {

constexpr int kF64Threads = 128;
constexpr int kF64Warps = kF64Threads / 32;

__device__ __forceinline__ int wrap_cell1(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

__device__ __forceinline__ double warp_sum_d(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// one pair energy of the trial (NEW) or the accepted state into the sum and the inf/NaN flags
template <bool NEW>
__device__ __forceinline__ void add_state(double u, double& e, int& f)
{
    if (isnan(u)) f |= NEW ? F_NEW_NAN : F_OLD_NAN;
    else if (isinf(u)) f |= NEW ? F_NEW_INF : F_OLD_INF;
    else e += NEW ? u : -u;
}

template <bool PHILOX>
__global__ void __launch_bounds__(kF64Threads, 4) fp64_chain_kernel(ChainArgs A)
{
    const long long t_start = clock64();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    DevSys& G = *A.sys[blockIdx.x];
    __shared__ __align__(16) DevSys Ssh;
    for (int w = tid; w < (int)(sizeof(DevSys) / 8); w += kF64Threads)
        reinterpret_cast<unsigned long long*>(&Ssh)[w] = reinterpret_cast<const unsigned long long*>(&G)[w];
    __shared__ MoveShared ms;
    __shared__ double red_p[kF64Warps], red_r[kF64Warps];
    __shared__ int red_f[kF64Warps];
    __shared__ int sh_acc, sh_stop, sh_up;
    __shared__ unsigned long long sh_t0;
    extern __shared__ __align__(16) unsigned char f64_smem[];
    __syncthreads();
    const DevSys& S = Ssh;
    const int K = (S.flags & SYS_EWALD) ? S.K : 0;
    double2* dq = reinterpret_cast<double2*>(f64_smem); // this move's change of Q(k)
    // per group, molecular moves: bit 0 the trial state's mass centres lie beyond the group
    // cutoff, bit 1 the accepted state's
    uint8_t* gcut = f64_smem + (size_t)K * sizeof(double2);

    // changes of Q(k) an FP32 chain left pending go into the FP64 master first (as fold_q_kernel
    // folds them), so that the phases below read Q as the chain holds it
    for (int k = tid; k < K; k += kF64Threads) {
        float2 pe = S.qpend[k];
        if (S.q_valid) {
            const float2 d = S.qdlt[k];
            pe.x += d.x;
            pe.y += d.y;
        }
        if (pe.x != 0.f || pe.y != 0.f) {
            double2 q = S.Q[k];
            q.x += (double)pe.x;
            q.y += (double)pe.y;
            S.Q[k] = q;
        }
        S.qpend[k] = make_float2(0.f, 0.f);
    }

    const long long nmoves = A.n_moves ? A.n_moves[blockIdx.x] : A.moves;
    const long long poff = A.prop_off ? A.prop_off[blockIdx.x] : 0;
    const uint32_t sys_id = A.sys_ids ? A.sys_ids[blockIdx.x] : blockIdx.x;
    const unsigned long long ctr0 = A.counters ? A.counters[blockIdx.x] + A.counter_base : A.counter_base;
    const bool molecular_sys = A.molecular ? (A.molecular[blockIdx.x] != 0) : false;
    const float dp_f = (float)(A.dp_sys ? A.dp_sys[blockIdx.x] : A.dp);
    const double dprot = A.dprot_sys ? A.dprot_sys[blockIdx.x] : A.dprot;
    const double twopi = 6.283185307179586476925286766559;

    // thread 0's running state
    double energy = sys_energy(S), sum_du = 0.0;
    double M[3] = {S.M[0], S.M[1], S.M[2]};
    unsigned long long n_acc = 0, n_mv = 0, n_pairs = 0, n_k = 0;
    if (tid == 0) {
        sh_t0 = global_ns();
        sh_up = 0;
    }
    int stop = 0;
    long long t = 0;
    for (; t < nmoves; t++) {
        // ---- the proposal and its trial positions (warp 0; prepare_move checks the caller's
        // proposals where it reads them: a bad index or kind ends the chain with FAU_ERR_ARG)
        if (warp == 0) {
            const Proposal p = PHILOX ? philox_proposal(S, ctr0 + (unsigned long long)t, sys_id, A.seed, dp_f, dprot,
                                                        molecular_sys)
                                      : load_proposal(A.props[poff + t]);
            prepare_move(S, ms, p, lane, nullptr, 0);
        }
        __syncthreads(); // B0: the move visible
        if (ms.stop) {
            stop = ms.stop;
            break;
        }
        const int kind = ms.kind, m = ms.m, first = ms.first;
        if (kind == FAU_MOVE_MOLECULAR) { // GroupCutoff of every other group, both states
            const int g = ms.index;
            for (int h = tid; h < S.n_groups; h += kF64Threads) {
                bool cut_o = false, cut_n = false;
                const double c2 = S.cut_g2g2 >= 0.0 ? group_cut2(S, g, h) : -1.0;
                if (h != g && c2 >= 0.0 && !(S.g_flags[h] & FAU_GROUP_ATOMIC)) {
                    const double cmh[3] = {S.g_cm[3 * h], S.g_cm[3 * h + 1], S.g_cm[3 * h + 2]};
                    const double cmo[3] = {S.g_cm[3 * g], S.g_cm[3 * g + 1], S.g_cm[3 * g + 2]};
                    cut_o = sqdist_d(S, cmo, cmh) >= c2;
                    cut_n = sqdist_d(S, ms.cm_new, cmh) >= c2;
                }
                gcut[h] = (uint8_t)((cut_n ? 1 : 0) | (cut_o ? 2 : 0));
            }
            __syncthreads();
        }
        if (kind != FAU_MOVE_NONE) {
            double ep = 0.0, er = 0.0;
            int f = 0;
            if (kind == FAU_MOVE_MOLECULAR) {
                const int g = ms.index;
                for (int j = tid; j < S.n; j += kF64Threads) {
                    const int gj = S.group_of[j];
                    if (gj == g) continue;
                    const int fc = gcut[gj];
                    const int tj = (int)(S.rec[j].w >> 24);
                    const double xj[3] = {S.x[j], S.y[j], S.z[j]};
                    for (int a = 0; a < m; a++) {
                        const int ti = (int)(ms.rec_old[a].w >> 24);
                        if (!(fc & 1)) add_state<true>(pair_u64(S, ti, tj, sqdist_d(S, ms.xn[a], xj)), ep, f);
                        if (!(fc & 2)) add_state<false>(pair_u64(S, ti, tj, sqdist_d(S, ms.xo[a], xj)), ep, f);
                    }
                }
            }
            else if (S.flags & SYS_CELLS) {
                // each state over the stencil of its own cell (GridOffsets3D, src/celllistimpl.cpp:
                // 15-31): every particle within the pair cutoff of a position lies in the stencil
                // of that position's cell
                const int i = first, ti = (int)(ms.rec_old[0].w >> 24);
                const int nbx = S.off_max[0] - S.off_min[0] + 1, nby = S.off_max[1] - S.off_min[1] + 1,
                          nbz = S.off_max[2] - S.off_min[2] + 1;
                const int cap = S.cap, cap_shift = __ffs(cap) - 1;
                const int per_state = (nbx * nby * nbz) << cap_shift;
                for (int s = tid; s < 2 * per_state; s += kF64Threads) {
                    const int st = s >= per_state ? 1 : 0; // 0: the trial state, 1: the accepted state
                    const int r = s - st * per_state, e = r >> cap_shift;
                    const int o[3] = {e % nbx + S.off_min[0], (e / nbx) % nby + S.off_min[1], e / (nbx * nby) + S.off_min[2]};
                    int c[3];
#pragma unroll
                    for (int d = 0; d < 3; d++) c[d] = wrap_cell1((st ? ms.cc_old[d] : ms.cc_new[d]) + o[d], S.cdim[d]);
                    const uint4 rj = S.cell_rec[(size_t)cell_index(S, c) * cap + (r & (cap - 1))];
                    if (rj.w == kEmptySlot) continue;
                    const int j = (int)(rj.w & 0xFFFFFFu);
                    if (j == i) continue;
                    const double xj[3] = {S.x[j], S.y[j], S.z[j]};
                    const double u = pair_u64(S, ti, (int)(rj.w >> 24), sqdist_d(S, st ? ms.xo[0] : ms.xn[0], xj));
                    if (st == 0) add_state<true>(u, ep, f);
                    else add_state<false>(u, ep, f);
                }
            }
            else {
                const int i = first, ti = (int)(ms.rec_old[0].w >> 24);
                for (int j = tid; j < S.n; j += kF64Threads) {
                    if (j == i) continue;
                    const int tj = (int)(S.rec[j].w >> 24);
                    const double xj[3] = {S.x[j], S.y[j], S.z[j]};
                    add_state<true>(pair_u64(S, ti, tj, sqdist_d(S, ms.xn[0], xj)), ep, f);
                    add_state<false>(pair_u64(S, ti, tj, sqdist_d(S, ms.xo[0], xj)), ep, f);
                }
            }
            if (K) {
                for (int k = tid; k < K; k += kF64Threads) {
                    int nx, ny, nz;
                    kn_unpack(S.kn[k], nx, ny, nz);
                    const double kx = twopi * ((double)nx / S.L[0]), ky = twopi * ((double)ny / S.L[1]),
                                 kz = twopi * ((double)nz / S.L[2]);
                    double dx = 0.0, dy = 0.0;
                    for (int a = 0; a < m; a++) {
                        const double q = S.itype_qd[ms.rec_old[a].w >> 24];
                        const double pn = (kx * ms.xn[a][0] + ky * ms.xn[a][1]) + kz * ms.xn[a][2];
                        const double po = (kx * ms.xo[a][0] + ky * ms.xo[a][1]) + kz * ms.xo[a][2];
                        double sn, cn, so, co;
                        sincos(pn, &sn, &cn);
                        sincos(po, &so, &co);
                        dx += q * cn - q * co;
                        dy += q * sn - q * so;
                    }
                    dq[k] = make_double2(dx, dy);
                    const double2 Q = S.Q[k];
                    const double nq2 = (Q.x + dx) * (Q.x + dx) + (Q.y + dy) * (Q.y + dy);
                    const double oq2 = Q.x * Q.x + Q.y * Q.y;
                    er += S.Akd[k] * (nq2 - oq2);
                }
            }
            ep = warp_sum_d(ep);
            er = warp_sum_d(er);
            f = (int)__reduce_or_sync(0xffffffffu, (unsigned)f);
            if (lane == 0) {
                red_p[warp] = ep;
                red_r[warp] = er;
                red_f[warp] = f;
            }
        }
        __syncthreads(); // B1: the warp partials visible

        // ---- decision and commit (thread 0)
        if (tid == 0) {
            int accept = 0, st = 0;
            double du = 0.0;
            if (kind != FAU_MOVE_NONE) {
                double ep = 0.0, er = 0.0;
                int f = 0;
#pragma unroll
                for (int w = 0; w < kF64Warps; w++) {
                    ep += red_p[w];
                    er += red_r[w];
                    f |= red_f[w];
                }
                const double du_rec = K ? S.rec_pref * er : 0.0;
                double du_surf = 0.0;
                if (S.flags & SYS_SURFACE) {
                    double m2o = 0.0, m2n = 0.0;
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        const double mn = __dadd_rn(M[d], ms.dM[d]);
                        m2o = __dadd_rn(m2o, __dmul_rn(M[d], M[d]));
                        m2n = __dadd_rn(m2n, __dmul_rn(mn, mn));
                    }
                    du_surf = S.surf_pref * (m2n - m2o);
                }
                du = energy_change(ep + (du_rec + du_surf), f & F_NEW_INF, f & F_OLD_INF, f & F_NEW_NAN, f & F_OLD_NAN);
                const double x = du * S.beta_scale;
                if (isnan(x)) st = FAU_ERR_NAN; // metropolisCriterion throws: the launch ends before this move
                else accept = metropolis(x, ms.u) ? 1 : 0;
                if (!st) {
                    n_mv++;
                    n_pairs += 2ull * (unsigned long long)m * (unsigned long long)(S.n - m);
                    n_k += (unsigned long long)K * (unsigned long long)m;
                }
            }
            if (!st) {
                if (A.acc_out) A.acc_out[poff + t] = (uint8_t)accept;
                if (A.du_out) A.du_out[poff + t] = du;
            }
            if (accept) { // State::sync trial -> accepted: positions, records, cell list, mass centre
                n_acc++;
                sum_du += du;
                energy += du;
                if (S.flags & SYS_SURFACE) {
#pragma unroll
                    for (int d = 0; d < 3; d++) M[d] = __dadd_rn(M[d], ms.dM[d]);
                }
                for (int a = 0; a < m; a++) {
                    S.x[first + a] = ms.xn[a][0];
                    S.y[first + a] = ms.xn[a][1];
                    S.z[first + a] = ms.xn[a][2];
                    S.rec[first + a] = ms.rec_new[a];
                }
                if (kind == FAU_MOVE_MOLECULAR) {
                    const int g = ms.index;
#pragma unroll
                    for (int d = 0; d < 3; d++) S.g_cm[3 * g + d] = ms.cm_new[d];
                    S.g_cmrec[g] = ms.cmrec_new;
                }
                else if (S.flags & SYS_CELLS) {
                    const int i = first;
                    const uint4 rn = ms.rec_new[0];
                    const int co = ms.cell_old, cn = ms.cell_new;
                    const int so = S.slot_of[i];
                    if (co == cn) {
                        S.cell_rec[(size_t)co * S.cap + so] = rn;
                    }
                    else {
                        const int last = S.cell_cnt[co] - 1;
                        if (so != last) {
                            const uint4 mvd = S.cell_rec[(size_t)co * S.cap + last];
                            S.cell_rec[(size_t)co * S.cap + so] = mvd;
                            S.slot_of[mvd.w & 0xFFFFFFu] = so;
                        }
                        S.cell_rec[(size_t)co * S.cap + last] = make_uint4(0u, 0u, 0u, kEmptySlot);
                        S.cell_cnt[co] = last;
                        const int sn = S.cell_cnt[cn];
                        if (sn >= S.cap) {
                            // a full destination keeps the particle listed in its old cell: the move
                            // is committed and the launch ends after it; the host regrows the list
                            S.cell_rec[(size_t)co * S.cap + last] = rn;
                            S.slot_of[i] = last;
                            S.cell_cnt[co] = last + 1;
                            st = FAU_ERR_CAPACITY;
                        }
                        else {
                            S.cell_rec[(size_t)cn * S.cap + sn] = rn;
                            S.cell_cnt[cn] = sn + 1;
                            S.cell_of[i] = cn;
                            S.slot_of[i] = sn;
                        }
                    }
                }
            }
            sh_acc = accept;
            sh_stop = st;
            if (A.time_budget_ns && global_ns() - sh_t0 >= A.time_budget_ns) sh_up = 1;
        }
        __syncthreads(); // B2: the decision visible
        if (sh_acc && K) // each thread its own k-vectors, as it wrote d_k above
            for (int k = tid; k < K; k += kF64Threads) {
                double2 q = S.Q[k];
                const double2 d = dq[k];
                q.x += d.x;
                q.y += d.y;
                S.Q[k] = q;
            }
        if (sh_stop) {
            stop = sh_stop;
            if (stop == FAU_ERR_CAPACITY) t++; // committed
            break;
        }
        if (sh_up) { // the time budget is spent: the launch ends after move t
            t++;
            break;
        }
    }
    __syncthreads();
    if (tid == 0) {
        G.pair_evals += n_pairs;
        G.k_updates += n_k;
        G.moves += n_mv;
        G.accepted += n_acc;
        G.sum_du += sum_du;
        G.energy = energy;
        G.e_acc_hi = G.e_acc_lo = 0.f;
#pragma unroll
        for (int d = 0; d < 3; d++) G.M[d] = M[d];
        G.q_valid = 0;
        G.q_since = 0;
        if (stop) G.err = stop;
        G.consumed = t;
        G.cycles += (unsigned long long)(clock64() - t_start);
    }
}

template <bool PH>
cudaError_t launch_fp64_inst(const ChainArgs& a, int nblocks, int K, int n_groups, cudaStream_t st, bool prepare_only)
{
    // the dynamic allowance is raised on demand, never inside a stream capture: callers prepare first
    static size_t granted = 0;
    const size_t smem = fp64_smem_bytes(K, n_groups);
    if (smem > granted || granted == 0) {
        const cudaError_t e =
            cudaFuncSetAttribute(fp64_chain_kernel<PH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        granted = smem;
    }
    if (prepare_only) return cudaSuccess;
    fp64_chain_kernel<PH><<<nblocks, kF64Threads, smem, st>>>(a);
    return cudaGetLastError();
}

} // namespace

size_t fp64_smem_bytes(int K, int n_groups)
{
    return (size_t)(K > 0 ? K : 0) * sizeof(double2) + (((size_t)(n_groups > 0 ? n_groups : 0) + 15) & ~size_t(15));
}

cudaError_t prepare_fp64(int K, int n_groups, bool philox)
{
    return philox ? launch_fp64_inst<true>(ChainArgs{}, 0, K, n_groups, nullptr, true)
                  : launch_fp64_inst<false>(ChainArgs{}, 0, K, n_groups, nullptr, true);
}

cudaError_t launch_fp64(const ChainArgs& a, int nblocks, int K, int n_groups, bool philox, cudaStream_t st)
{
    return philox ? launch_fp64_inst<true>(a, nblocks, K, n_groups, st, false)
                  : launch_fp64_inst<false>(a, nblocks, K, n_groups, st, false);
}

} // namespace fau
