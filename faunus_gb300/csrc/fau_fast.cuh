// fau_fast.cuh -- the pipelined chain kernel for batches of single-atom-move
// systems (one CTA per chain).
//
// It performs the same Metropolis step as chain_kernel
// (MetropolisMonteCarlo::performMove, reference src/montecarlo.cpp:139-187, for
// AtomicTranslateRotate, src/move.cpp:225-240) with the same FP64 position
// arithmetic, but arranges the work so that little besides the energy change
// itself lies on a chain's serial path:
//
//   warp 0 (producer)    while the compute warps evaluate move t it commits
//                        nothing and waits on nothing: it prepares move t+1
//                        (FP64 trial position, fixed-point record, cells,
//                        phase tables, the cell stencils), loads the particle
//                        state of move t+2 and the cell-list entries the
//                        commit of move t+1 will rewrite.
//   warps 1..W (compute) Ewald dU over the k-vectors and pair dU over the
//                        union of the old and new 3x3x3 cell stencils, both
//                        states per record; the records are loaded before the
//                        Ewald loop so their latency hides behind it.
//   barrier              every thread then sums the warp partials in one
//                        fixed order and takes the same Metropolis decision,
//                        applies its own share of the Q(k) update, and goes on
//                        to move t+1; the producer commits move t.
//
// A second barrier is taken only when move t is accepted and move t+1 reads
// what its commit rewrites: the same particle (move t+1 is then prepared
// again), or a cell of move t+1's stencils.  Move data lives in three
// rotating shared-memory slots (t, t+1 and the one the producer fills), the
// warp partials in two.
#pragma once
#include "fau_chain.cuh"

namespace fau {

constexpr int kFastEntries = 64; // cells listed per move: union box (<= 4x4x4) or two stencils (<= 54)
constexpr int kFastRing = 64;    // host proposals staged in shared memory, refilled 32 at a time

enum : int { FC_SELF = 1, FC_CELLS = 2 };
constexpr int kFastUnsupported = -2; // proposal kind this kernel does not handle (FAU_MOVE_NONE is -1)
constexpr uint32_t kEntNew = 1u << 30, kEntOld = 1u << 31, kEntCell = kEntNew - 1u;

struct FastMove {
    int kind, i, cell_old, cell_new;
    int nue, conflict, cap_full, stop; // conflict: FC_* against the previous move
    int cc_o[3], cc_n[3];
    uint4 ro, rn;
    double xo[3], xn[3], dM[3];
    double u;
    float q, gx, gy, gz;
    uint32_t ent[kFastEntries]; // cell | kEntNew (trial state reads it) | kEntOld (accepted state)
};

// The move after next: its proposal (written by lane 0) and the moved particle's
// resident state, copied from global memory asynchronously one move early.
struct Ahead {
    uint4 rec;
    double x[3];
    double dr[3], u;
    int kind, i, cell, pad;
};

// cell-list state read ahead of a commit (asynchronous copies as well)
struct CommitPre {
    uint4 last;
    int so, cnt_o, cnt_n, pad;
};

// cp.async (global -> shared, completion tracked per commit group): the copies
// land while the issuing warp goes on working
__device__ __forceinline__ void cp_async(void* smem, const void* gmem, int bytes)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    if (bytes == 16) asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
    else if (bytes == 8) asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
    else asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait()
{
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

template <bool PHILOX>
__device__ __forceinline__ void fast_proposal(const DevSys& S, const ChainArgs& A, const fau_proposal* ring, long long s,
                                              unsigned long long ctr0, uint32_t sys_id, Ahead& a)
{
    if (PHILOX) {
        const Proposal p = philox_proposal(S, ctr0 + (unsigned long long)s, sys_id, A.seed, A.dp, A.dprot, false);
        a.kind = p.kind;
        a.i = p.index;
#pragma unroll
        for (int d = 0; d < 3; d++) a.dr[d] = p.dr[d];
        a.u = p.u;
    }
    else {
        const fau_proposal& f = ring[s % kFastRing];
        a.kind = (f.kind == FAU_MOVE_ATOMIC || f.kind == FAU_MOVE_NONE) ? f.kind : kFastUnsupported;
        a.i = f.index;
#pragma unroll
        for (int d = 0; d < 3; d++) a.dr[d] = f.dr[d];
        a.u = f.u;
    }
}

// start the copies of the moved particle's state (lane 0; complete after the next wait)
__device__ __forceinline__ void fast_load(const DevSys& S, Ahead& a)
{
    if (a.kind == FAU_MOVE_ATOMIC) {
        const int i = a.i;
        cp_async(&a.x[0], S.x + i, 8);
        cp_async(&a.x[1], S.y + i, 8);
        cp_async(&a.x[2], S.z + i, 8);
        cp_async(&a.rec, S.rec + i, 16);
        if (S.flags & SYS_CELLS) cp_async(&a.cell, S.cell_of + i, 4);
    }
}

// start the copies of the cell-list entries a commit of `m` reads (lane 0)
__device__ __forceinline__ void fast_commit_loads(const DevSys& S, const FastMove& m, CommitPre& c)
{
    if ((S.flags & SYS_CELLS) && m.kind == FAU_MOVE_ATOMIC) {
        cp_async(&c.so, S.slot_of + m.i, 4);
        if (m.cell_old != m.cell_new) {
            cp_async(&c.cnt_o, S.cell_cnt + m.cell_old, 4);
            cp_async(&c.cnt_n, S.cell_cnt + m.cell_new, 4);
        }
    }
}

__device__ __forceinline__ int wrap_cell(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

// Producer warp: trial position, record, cells, phase tables and cell entries of
// the move staged in `m`; `prev` is the move evaluated just before it.
static __device__ __noinline__ void fast_prepare(const DevSys& S, FastMove& m, const Ahead& a, const FastMove* prev,
                                                 int lane, float2* T, int nc, const double* itq)
{
    const int TS = 2 * nc + 1;
    const bool cells = (S.flags & SYS_CELLS) != 0;
    if (lane == 0) {
        const int kind = a.kind;
        m.kind = kind == kFastUnsupported ? FAU_MOVE_NONE : kind;
        m.i = a.i;
        m.u = a.u;
        m.stop = kind == kFastUnsupported ? FAU_ERR_ARG : 0; // molecular proposal: not handled by this kernel
        m.cap_full = 0;
        m.nue = 0;
        if (kind == FAU_MOVE_ATOMIC) {
            double xo[3], xn[3];
#pragma unroll
            for (int d = 0; d < 3; d++) {
                xo[d] = a.x[d];
                xn[d] = boundary1(__dadd_rn(xo[d], a.dr[d]), S.L[d], S.half[d], S.inv[d]);
            }
            const uint4 ro = a.rec;
            m.ro = ro;
            m.cell_old = a.cell;
            const uint4 rn = make_uint4(to_fixed(xn[0], S.fx_scale[0]), to_fixed(xn[1], S.fx_scale[1]),
                                        to_fixed(xn[2], S.fx_scale[2]), ro.w);
            const double q = itq[ro.w >> 24];
            m.rn = rn;
            m.q = (float)q;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                m.xo[d] = xo[d];
                m.xn[d] = xn[d];
                m.dM[d] = __dmul_rn(q, __dsub_rn(xn[d], xo[d]));
            }
            const float3 g = min_image_frac(S, xn, xo);
            m.gx = g.x;
            m.gy = g.y;
            m.gz = g.z;
            if (cells) {
                const int co = a.cell;
                m.cc_o[0] = co % S.cdim[0];
                m.cc_o[1] = (co / S.cdim[0]) % S.cdim[1];
                m.cc_o[2] = co / (S.cdim[0] * S.cdim[1]);
                int c[3];
                cell_coords(S, xn, rn, c);
                m.cc_n[0] = c[0];
                m.cc_n[1] = c[1];
                m.cc_n[2] = c[2];
                m.cell_new = cell_index(S, c);
            }
            else {
                m.cell_old = m.cell_new = 0;
            }
        }
        else {
            m.i = -1;
            m.cell_old = m.cell_new = -1;
        }
    }
    __syncwarp();
    if (m.kind != FAU_MOVE_ATOMIC) {
        if (lane == 0) m.conflict = 0;
        __syncwarp();
        return;
    }
    // phase tables: per axis, mid = e^{i n (phi + pi g)} and h = e^{i n pi g}, n = -nc..nc
    if (T) {
        const uint4 ro = m.ro;
        const float gx = m.gx, gy = m.gy, gz = m.gz;
        for (int e = lane; e < 3 * (nc + 1); e += 32) {
            const int ax = e / (nc + 1), n = e - ax * (nc + 1);
            const uint32_t u = ax == 0 ? ro.x : (ax == 1 ? ro.y : ro.z);
            const float g = ax == 0 ? gx : (ax == 1 ? gy : gz);
            float s, c;
            sincospif((float)n * g, &s, &c);
            const float2 h = make_float2(c, s);
            const float2 mid = cmul(phase_exact((uint32_t)n * u), h);
            float2* row = T + 2 * ax * TS;
            row[nc + n] = mid;
            row[nc - n] = make_float2(mid.x, -mid.y);
            row[TS + nc + n] = h;
            row[TS + nc - n] = make_float2(h.x, -h.y);
        }
    }
    bool hit = false;
    if (cells) {
        int cco[3], ccn[3], df[3], lo[3], w[3];
        bool uni = true;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            cco[d] = m.cc_o[d];
            ccn[d] = m.cc_n[d];
            const int n = S.cdim[d];
            int v = ccn[d] - cco[d];
            if (2 * v > n) v -= n;
            else if (2 * v < -n) v += n;
            df[d] = v;
            if (v < -1 || v > 1 || n < 3 + abs(v)) uni = false;
            lo[d] = cco[d] + min(v, 0) - 1;
            w[d] = 3 + abs(v);
        }
        const int pc_o = prev && prev->kind == FAU_MOVE_ATOMIC ? prev->cell_old : -1;
        const int pc_n = prev && prev->kind == FAU_MOVE_ATOMIC ? prev->cell_new : -1;
        int nue;
        if (uni) { // one box holding both stencils; each cell flags the states whose stencil contains it
            nue = w[0] * w[1] * w[2];
            for (int e = lane; e < nue; e += 32) {
                const int ex = e % w[0], ey = (e / w[0]) % w[1], ez = e / (w[0] * w[1]);
                const int o[3] = {lo[0] + ex, lo[1] + ey, lo[2] + ez};
                bool in_o = true, in_n = true;
                int c[3];
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    in_o = in_o && abs(o[d] - cco[d]) <= 1;
                    in_n = in_n && abs(o[d] - (cco[d] + df[d])) <= 1;
                    c[d] = wrap_cell(o[d], S.cdim[d]);
                }
                const int cell = cell_index(S, c);
                hit = hit || cell == pc_o || cell == pc_n;
                m.ent[e] = (uint32_t)cell | (in_n ? kEntNew : 0u) | (in_o ? kEntOld : 0u);
            }
        }
        else { // the two neighbour stencils listed separately (GridOffsets3D src/celllistimpl.cpp:15-31)
            const int nbx = S.off_max[0] - S.off_min[0] + 1, nby = S.off_max[1] - S.off_min[1] + 1,
                      nbz = S.off_max[2] - S.off_min[2] + 1;
            const int nb = nbx * nby * nbz;
            nue = 2 * nb;
            for (int e = lane; e < nue; e += 32) {
                const int st = e >= nb ? 1 : 0, r = e - st * nb;
                const int o[3] = {r % nbx + S.off_min[0], (r / nbx) % nby + S.off_min[1], r / (nbx * nby) + S.off_min[2]};
                int c[3];
#pragma unroll
                for (int d = 0; d < 3; d++) c[d] = wrap_cell((st ? ccn[d] : cco[d]) + o[d], S.cdim[d]);
                const int cell = cell_index(S, c);
                hit = hit || cell == pc_o || cell == pc_n;
                m.ent[e] = (uint32_t)cell | (st ? kEntNew : kEntOld);
            }
        }
        if (lane == 0) m.nue = nue;
    }
    hit = __any_sync(0xffffffffu, hit);
    if (lane == 0) {
        const bool self = prev && prev->kind == FAU_MOVE_ATOMIC && prev->i == m.i;
        m.conflict = (self ? FC_SELF : 0) | (hit ? FC_CELLS : 0);
    }
    __syncwarp();
}

struct PairOut {
    float u, mag;
    int flags; // F_* bits of this state
};

// one state of one pair (a single call site keeps the kernel's code small)
static __device__ __noinline__ PairOut fast_pair_state(const DevSys& S, PairF p, int pidx, float r2, const double* xi,
                                                        int j, const double* xj, bool is_new)
{
    bool inf = false, nan = false;
    float mag = 0.f;
    const float u = pair_u32(S, p, pidx, r2, xi, j, inf, nan, mag, xj);
    PairOut o;
    o.u = u;
    o.mag = mag;
    o.flags = is_new ? ((inf ? F_NEW_INF : 0) | (nan ? F_NEW_NAN : 0)) : ((inf ? F_OLD_INF : 0) | (nan ? F_OLD_NAN : 0));
    return o;
}

// Metropolis decision shared by every thread: FP32 unless the exponential is
// within 1e-4 of u (or an infinity, NaN or the surface term is involved), then
// the exact FP64 form metropolisCriterion (src/montecarlo.cpp:17-34) on the
// getEnergyChange value (src/montecarlo.cpp:193-209).  Returns accept; sets
// nan_stop for a NaN energy change.
__device__ __forceinline__ bool fast_decide(FF s, int flags, double du_surf, bool surface, double beta, float beta_f,
                                            double u, bool& nan_stop)
{
    nan_stop = false;
    if (flags == 0 && !surface) {
        const float xf = (s.hi + s.lo) * beta_f;
        if (xf <= 0.f) return true;
        const float ef = __expf(-xf);
        if (ef > 1e-30f) {
            const float uf = (float)u;
            if (uf < ef * 0.9999f) return true;
            if (uf > ef * 1.0001f) return false;
        }
        else if (u > 1e-29) {
            return false;
        }
    }
    const double du = energy_change(ff_value(s) + du_surf, flags & F_NEW_INF, flags & F_OLD_INF, flags & F_NEW_NAN,
                                    flags & F_OLD_NAN);
    const double x = du * beta;
    if (isnan(x)) {
        nan_stop = true;
        return false;
    }
    return metropolis(x, u);
}

template <int NWC, bool PHILOX>
__global__ void __launch_bounds__(32 * (NWC + 1), 4) fast_chain_kernel(ChainArgs A)
{
    constexpr int NT = 32 * (NWC + 1), NTC = 32 * NWC;
    DevSys& S = *A.sys[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const bool producer = warp == 0;
    const int ctid = tid - 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int K = (S.flags & SYS_EWALD) ? S.K : 0;
    const int nc = S.knc;
    const int TS = 2 * nc + 1;
    const int nt = S.nt;
    float4* kq = reinterpret_cast<float4*>(smem_raw); // {Q.x, Q.y, pending.x, pending.y} (FP32 copy + accepted, unflushed)
    float2* dlt = reinterpret_cast<float2*>(kq + K);  // this move's change of Q(k)
    int2* kaf = reinterpret_cast<int2*>(dlt + K);     // {(nx+nc) | (ny+nc)<<8 | (nz+nc)<<16, (2 pi lB / V) A_k}
    float2* tabs = reinterpret_cast<float2*>(kaf + K); // 3 slots x 6 rows x TS phase tables
    PairF* pt = reinterpret_cast<PairF*>(tabs + 3 * 6 * TS);

    __shared__ FastMove mvb[3];
    __shared__ Ahead ahs[2];       // move s: ahs[s & 1]
    __shared__ CommitPre cps[2];   // move s: cps[s & 1]
    __shared__ FF red_a[2][NWC];
    __shared__ int red_f[2][NWC];
    __shared__ double itq[kMaxITypes];
    __shared__ fau_proposal ring[PHILOX ? 1 : kFastRing];
    __shared__ unsigned long long red_u[NWC][2];

    const float rec_pref_f = (float)S.rec_pref;
    for (int k = tid; k < K; k += NT) {
        const double2 q = S.Q[k];
        kq[k] = make_float4((float)q.x, (float)q.y, 0.f, 0.f);
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        kaf[k] = make_int2((nx + nc) | ((ny + nc) << 8) | ((nz + nc) << 16), __float_as_int(rec_pref_f * S.Ak[k]));
    }
    for (int t = tid; t < nt * nt; t += NT) pt[t] = S.pair[t];
    if (tid < nt) itq[tid] = S.itype_qd[tid];

    const long long nmoves = A.n_moves ? A.n_moves[blockIdx.x] : A.moves;
    const long long poff = A.prop_off ? A.prop_off[blockIdx.x] : 0;
    const uint32_t sys_id = A.sys_ids ? A.sys_ids[blockIdx.x] : blockIdx.x;
    const unsigned long long ctr0 = A.counters ? A.counters[blockIdx.x] + A.counter_base : A.counter_base;
    const bool cells = (S.flags & SYS_CELLS) != 0;
    const bool surface = (S.flags & SYS_SURFACE) != 0;
    const int cap = S.cap;
    const int cap_shift = cells ? __ffs(cap) - 1 : 0;
    const double beta = S.beta_scale, surf_pref = S.surf_pref;
    const float beta_f = (float)beta;
    double M[3] = {S.M[0], S.M[1], S.M[2]};

    // proposals [s0, s0 + 32) into their ring slots (host proposals)
    auto ring_fill = [&](long long s0) {
        const long long e = s0 + 32 < nmoves ? s0 + 32 : nmoves;
        if (e <= s0) return;
        const int words = (int)(e - s0) * (int)(sizeof(fau_proposal) / 8);
        const unsigned long long* src = reinterpret_cast<const unsigned long long*>(A.props + poff + s0);
        unsigned long long* dst = reinterpret_cast<unsigned long long*>(ring + (s0 % kFastRing));
        for (int w = lane; w < words; w += 32) dst[w] = src[w];
    };

    unsigned long long n_acc = 0, n_mv = 0, n_pairs = 0, n_k = 0;
    double energy = S.energy, sum_du = 0.0;
    int since_flush = 0;

    if (producer) {
        if (!PHILOX) {
            ring_fill(0);
            ring_fill(32);
            __syncwarp();
        }
        if (lane == 0 && nmoves > 0) {
            fast_proposal<PHILOX>(S, A, ring, 0, ctr0, sys_id, ahs[0]);
            fast_load(S, ahs[0]);
            cp_async_commit();
            cp_async_wait<0>();
        }
        __syncwarp();
        if (nmoves > 0) fast_prepare(S, mvb[0], ahs[0], nullptr, lane, K ? tabs : nullptr, nc, itq);
        if (lane == 0) {
            if (nmoves > 1) {
                fast_proposal<PHILOX>(S, A, ring, 1, ctr0, sys_id, ahs[1]);
                fast_load(S, ahs[1]);
            }
            fast_commit_loads(S, mvb[0], cps[0]);
            cp_async_commit();
        }
    }
    __syncthreads();

    int prev_accept = 0, stop = 0;
    long long consumed = nmoves;
    for (long long t = 0; t < nmoves; t++) {
        const int b = (int)(t % 3);
        FastMove& m = mvb[b];
        if (m.stop) {
            stop = m.stop;
            consumed = t;
            break;
        }
        const int kind = m.kind;
        const int rb = (int)(t & 1);
        if (producer) {
            CommitPre& cp = cps[t & 1];
            if (lane == 0) {
                cp_async_wait<0>(); // Ahead of move t+1, commit counts of move t
                if (kind == FAU_MOVE_ATOMIC && cells) {
                    // read before move t-1's commit: read again if that commit touched them
                    if (prev_accept && m.conflict) {
                        fast_commit_loads(S, m, cp);
                        cp_async_commit();
                        cp_async_wait<0>();
                    }
                    if (m.cell_old != m.cell_new) {
                        const int last = cp.cnt_o - 1;
                        if (last >= 0 && last < cap && last != cp.so)
                            cp_async(&cp.last, S.cell_rec + (size_t)m.cell_old * cap + last, 16);
                        m.cap_full = cp.cnt_n >= cap ? 1 : 0;
                    }
                }
                cp_async_commit(); // group 1: the record that fills the old cell's hole
            }
            if (!PHILOX && (t & 31) == 0 && t >= 32) ring_fill(t + 32);
            if (t + 1 < nmoves) {
                const FastMove& pm = mvb[(t + 2) % 3]; // move t-1
                Ahead& an = ahs[(t + 1) & 1];
                if (lane == 0 && t >= 1 && prev_accept && pm.kind == FAU_MOVE_ATOMIC && an.kind == FAU_MOVE_ATOMIC &&
                    an.i == pm.i) { // copied before move t-1's commit: take the committed state
#pragma unroll
                    for (int d = 0; d < 3; d++) an.x[d] = pm.xn[d];
                    an.rec = pm.rn;
                    an.cell = pm.cell_new;
                }
                __syncwarp();
                fast_prepare(S, mvb[(t + 1) % 3], an, &m, lane, K ? tabs + ((t + 1) % 3) * 6 * TS : nullptr, nc, itq);
                if (lane == 0) {
                    if (t + 2 < nmoves) {
                        Ahead& a2 = ahs[t & 1];
                        fast_proposal<PHILOX>(S, A, ring, t + 2, ctr0, sys_id, a2);
                        fast_load(S, a2);
                    }
                    fast_commit_loads(S, mvb[(t + 1) % 3], cps[(t + 1) & 1]);
                }
            }
            if (lane == 0) cp_async_commit(); // group 2: Ahead of move t+2, commit counts of move t+1
        }
        else if (kind == FAU_MOVE_ATOMIC) {
            const int i = m.i;
            const uint4 ro = m.ro, rn = m.rn;
            const int ti = rn.w >> 24;
            // all-pairs mode: the previous move's particle may not be in memory yet
            int pi = -1;
            uint4 prn = make_uint4(0, 0, 0, 0);
            const double* pxn = nullptr;
            if (!cells && prev_accept && t >= 1) {
                const FastMove& pm = mvb[(t + 2) % 3];
                if (pm.kind == FAU_MOVE_ATOMIC) {
                    pi = pm.i;
                    prn = pm.rn;
                    pxn = pm.xn;
                }
            }
            const int n_items = cells ? (m.nue << cap_shift) : S.n;
            auto load_item = [&](int it, uint4& rj, uint32_t& ent) {
                if (cells) {
                    ent = m.ent[it >> cap_shift];
                    rj = S.cell_rec[(size_t)(ent & kEntCell) * cap + (it & (cap - 1))];
                }
                else {
                    ent = kEntNew | kEntOld;
                    rj = S.rec[it];
                }
            };
            uint4 r0 = make_uint4(0, 0, 0, kEmptySlot), r1 = r0;
            uint32_t e0 = 0, e1 = 0;
            if (ctid < n_items) load_item(ctid, r0, e0);
            if (ctid + NTC < n_items) load_item(ctid + NTC, r1, e1);

            // ---- Ewald: one k-vector per thread and step, two independent accumulators
            FF acc0{0.f, 0.f}, acc1{0.f, 0.f};
            if (K) {
                const float2* Tb = tabs + b * 6 * TS;
                const float f0 = 2.f * m.q;
                auto ewald_k = [&](int k, FF& acc) {
                    const int2 ka = kaf[k];
                    const int ix = ka.x & 0xff, iy = (ka.x >> 8) & 0xff, iz = ka.x >> 16;
                    const float2 mid = cmul(cmul(Tb[ix], Tb[2 * TS + iy]), Tb[4 * TS + iz]);
                    const float2 hxy = cmul(Tb[TS + ix], Tb[3 * TS + iy]);
                    const float2 hz = Tb[5 * TS + iz];
                    const float f = f0 * fmaf(hxy.x, hz.y, hxy.y * hz.x); // 2 q sin(D/2)
                    const float2 d = make_float2(-f * mid.y, f * mid.x);
                    dlt[k] = d;
                    const float4 qq = kq[k];
                    const float qx = qq.x + qq.z, qy = qq.y + qq.w;
                    const float cross = 2.f * fmaf(qx, d.x, qy * d.y);
                    const float dd = fmaf(d.x, d.x, d.y * d.y);
                    ff_add(acc, __int_as_float(ka.y) * (cross + dd));
                };
                int k = ctid;
                for (; k + NTC < K; k += 2 * NTC) {
                    ewald_k(k, acc0);
                    ewald_k(k + NTC, acc1);
                }
                if (k < K) ewald_k(k, acc0);
                n_k += (unsigned long long)((K - ctid + NTC - 1) / NTC);
            }
            FF accp = ff_sum(acc0, acc1);
            int flags = 0;

            // ---- pairs
            for (int r = 0;; r++) {
                const int it = ctid + r * NTC;
                if (it >= n_items) break;
                uint4 rj;
                uint32_t ent;
                if (r == 0) {
                    rj = r0;
                    ent = e0;
                }
                else if (r == 1) {
                    rj = r1;
                    ent = e1;
                }
                else {
                    load_item(it, rj, ent);
                }
                if (rj.w == kEmptySlot) continue;
                int j = (int)(rj.w & 0xFFFFFFu);
                if (!cells) j = it;
                if (j == i) continue;
                const double* xj = nullptr;
                if (j == pi) {
                    rj = prn;
                    xj = pxn;
                }
                const int pidx = ti * nt + (int)(rj.w >> 24);
                const PairF p = pt[pidx];
                float un = 0.f, uo = 0.f;
                for (int st = 0; st < 2; st++) {
                    if (!(ent & (st ? kEntOld : kEntNew))) continue;
                    const PairOut o = fast_pair_state(S, p, pidx, r2_fixed(S, st ? ro : rn, rj), st ? m.xo : m.xn, j,
                                                      xj, st == 0);
                    if (st) uo = o.u;
                    else un = o.u;
                    flags |= o.flags;
                    n_pairs++;
                }
                ff_add(accp, un - uo);
            }
            float sc_unused = 0.f;
            FF b_unused{0.f, 0.f};
            warp_reduce(accp, b_unused, sc_unused, flags, false);
            if (lane == 0) {
                red_a[rb][warp - 1] = accp;
                red_f[rb][warp - 1] = flags;
            }
        }
        __syncthreads(); // B1

        // ---- decision, identical in every thread
        int accept = 0;
        bool nan_stop = false;
        double du_surf = 0.0;
        FF s{0.f, 0.f};
        int fl = 0;
        if (kind == FAU_MOVE_ATOMIC) {
#pragma unroll
            for (int w = 0; w < NWC; w++) {
                s = ff_sum(s, red_a[rb][w]);
                fl |= red_f[rb][w];
            }
            if (surface) {
                double m2o = 0.0, m2n = 0.0;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    const double mn = __dadd_rn(M[d], m.dM[d]);
                    m2o = __dadd_rn(m2o, __dmul_rn(M[d], M[d]));
                    m2n = __dadd_rn(m2n, __dmul_rn(mn, mn));
                }
                du_surf = surf_pref * (m2n - m2o);
            }
            accept = fast_decide(s, fl, du_surf, surface, beta, beta_f, m.u, nan_stop) ? 1 : 0;
        }
        if (nan_stop) {
            stop = FAU_ERR_NAN;
            consumed = t;
            break;
        }
        if (producer && lane == 0) {
            double du = 0.0;
            if (kind == FAU_MOVE_ATOMIC) {
                if (accept || A.du_out)
                    du = energy_change(ff_value(s) + du_surf, fl & F_NEW_INF, fl & F_OLD_INF, fl & F_NEW_NAN,
                                       fl & F_OLD_NAN);
                n_mv++;
                if (accept) {
                    n_acc++;
                    sum_du += du;
                    energy += du;
                }
            }
            if (A.acc_out) A.acc_out[poff + t] = (uint8_t)accept;
            if (A.du_out) A.du_out[poff + t] = du;
        }
        if (accept) {
            if (surface) {
#pragma unroll
                for (int d = 0; d < 3; d++) M[d] = __dadd_rn(M[d], m.dM[d]);
            }
            if (!producer && K) { // this thread's share of Q(k) += dQ(k); FP32 pending -> FP64 master every N accepts
                const bool flush = ++since_flush == kFlushAccepts;
                if (flush) since_flush = 0;
                for (int k = ctid; k < K; k += NTC) {
                    float4 qq = kq[k];
                    const float2 d = dlt[k];
                    qq.z += d.x;
                    qq.w += d.y;
                    if (flush) {
                        double2 q = S.Q[k];
                        q.x += (double)qq.z;
                        q.y += (double)qq.w;
                        S.Q[k] = q;
                        qq = make_float4((float)q.x, (float)q.y, 0.f, 0.f);
                    }
                    kq[k] = qq;
                }
            }
            if (producer && lane == 0) { // commit (State::sync trial -> accepted): positions, record, cell list
                cp_async_wait<1>();
                const CommitPre& cp_cur = cps[t & 1];
                const int i = m.i;
                S.x[i] = m.xn[0];
                S.y[i] = m.xn[1];
                S.z[i] = m.xn[2];
                S.rec[i] = m.rn;
                const bool sane = cp_cur.so >= 0 && cp_cur.so < cap &&
                                  (m.cell_old == m.cell_new ||
                                   (cp_cur.cnt_o >= 1 && cp_cur.cnt_o <= cap && cp_cur.cnt_n >= 0));
                if (cells && !sane) {
                    S.err = FAU_ERR_STATE; // inconsistent cell list: leave it untouched
                }
                else if (cells) {
                    const int co = m.cell_old, cn = m.cell_new;
                    if (co == cn || m.cap_full) {
                        // a full destination keeps the particle listed in its old cell: the host regrows the list
                        S.cell_rec[(size_t)co * cap + cp_cur.so] = m.rn;
                    }
                    else {
                        const int last = cp_cur.cnt_o - 1;
                        if (cp_cur.so != last) {
                            S.cell_rec[(size_t)co * cap + cp_cur.so] = cp_cur.last;
                            S.slot_of[cp_cur.last.w & 0xFFFFFFu] = cp_cur.so;
                        }
                        S.cell_rec[(size_t)co * cap + last] = make_uint4(0u, 0u, 0u, kEmptySlot);
                        S.cell_cnt[co] = last;
                        S.cell_rec[(size_t)cn * cap + cp_cur.cnt_n] = m.rn;
                        S.cell_cnt[cn] = cp_cur.cnt_n + 1;
                        S.cell_of[i] = cn;
                        S.slot_of[i] = cp_cur.cnt_n;
                    }
                }
            }
            if (m.cap_full) {
                stop = FAU_ERR_CAPACITY;
                consumed = t + 1;
                break;
            }
        }
        // ---- the next move reads what this commit rewrote: make it visible (and re-prepare a same-particle move)
        const int nconf = (accept && t + 1 < nmoves) ? mvb[(t + 1) % 3].conflict : 0;
        if (nconf) {
            if (producer && (nconf & FC_SELF)) {
                FastMove& nm = mvb[(t + 1) % 3];
                Ahead& an = ahs[(t + 1) & 1];
                if (lane == 0) {
                    cp_async_wait<0>();
                    fast_proposal<PHILOX>(S, A, ring, t + 1, ctr0, sys_id, an);
                    fast_load(S, an);
                    cp_async_commit();
                    cp_async_wait<0>();
                }
                __syncwarp();
                fast_prepare(S, nm, an, &m, lane, K ? tabs + ((t + 1) % 3) * 6 * TS : nullptr, nc, itq);
                if (lane == 0) {
                    fast_commit_loads(S, nm, cps[(t + 1) & 1]);
                    cp_async_commit();
                }
            }
            __syncthreads(); // B2
        }
        prev_accept = accept;
    }
    if (producer && lane == 0) cp_async_wait<0>();

    // everything pending into the FP64 master Q
    if (!producer) {
        for (int k = ctid; k < K; k += NTC) {
            const float4 qq = kq[k];
            if (qq.z != 0.f || qq.w != 0.f) {
                double2 q = S.Q[k];
                q.x += (double)qq.z;
                q.y += (double)qq.w;
                S.Q[k] = q;
            }
        }
    }
    unsigned long long pa = n_pairs, kb = n_k;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        pa += __shfl_xor_sync(0xffffffffu, pa, o);
        kb += __shfl_xor_sync(0xffffffffu, kb, o);
    }
    if (!producer && lane == 0) {
        red_u[warp - 1][0] = pa;
        red_u[warp - 1][1] = kb;
    }
    __syncthreads();
    if (tid == 0) {
        unsigned long long sp = 0, sk = 0;
        for (int w = 0; w < NWC; w++) {
            sp += red_u[w][0];
            sk += red_u[w][1];
        }
        S.pair_evals += sp;
        S.k_updates += sk;
        S.moves += n_mv;
        S.accepted += n_acc;
        S.sum_du += sum_du;
        S.energy = energy;
#pragma unroll
        for (int d = 0; d < 3; d++) S.M[d] = M[d];
        if (stop) S.err = stop;
        S.consumed = consumed;
    }
}

// dynamic shared memory of the pipelined kernel for K k-vectors, table size nc
__host__ __device__ inline size_t fast_smem_bytes(int K, int nc)
{
    return (size_t)K * (sizeof(float4) + sizeof(float2) + sizeof(int2)) + (size_t)3 * 6 * (2 * nc + 1) * sizeof(float2) +
           (size_t)kMaxITypes * kMaxITypes * sizeof(PairF);
}

template <int NWC, bool PH>
cudaError_t launch_fast_inst(const ChainArgs& a, int nblocks, int K, int nc, cudaStream_t st, bool prepare_only)
{
    // the dynamic allowance is raised on demand, never inside a stream capture: callers prepare first
    static size_t granted = 0;
    const size_t smem = fast_smem_bytes(K, nc);
    if (smem > granted || granted == 0) {
        cudaError_t e = cudaFuncSetAttribute(fast_chain_kernel<NWC, PH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        granted = smem;
    }
    if (prepare_only) return cudaSuccess;
    fast_chain_kernel<NWC, PH><<<nblocks, 32 * (NWC + 1), smem, st>>>(a);
    return cudaGetLastError();
}

} // namespace fau
