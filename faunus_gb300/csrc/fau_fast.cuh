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
constexpr int kFastFlushAccepts = 256; // FP32 pending Q deltas flushed to the FP64 master every N accepts
constexpr int kFastStagePerThread = 4; // pair records staged in shared memory per compute thread: two
                                       // half-rounds of two, one filling while the other is evaluated
__host__ __device__ constexpr int fast_stage_items(int nwc) { return kFastStagePerThread * 32 * nwc; }

enum : int { FC_SELF = 1, FC_CELLS = 2 };
constexpr int kFastUnsupported = -2; // proposal kind this kernel does not handle (FAU_MOVE_NONE is -1)
constexpr uint32_t kEntNew = 1u << 30, kEntOld = 1u << 31, kEntCell = kEntNew - 1u;

struct FastMove {
    int kind, i, cell_old, cell_new;
    int nue, conflict, cap_full, stop; // conflict: FC_* against the previous move
    int cc_o[3], cc_n[3];
    int uni, lo[3], w[3], df[3];       // cell entries: union box (uni) or the two stencils
    float g[3];                        // displacement / L (phase tables)
    uint4 ro, rn;
    double xo[3], xn[3], dM[3];
    double u, du_surf; // du_surf: Ewald surface-term change, computed by the producer before the barrier
    float uf, q;
    uint32_t ent[kFastEntries]; // cell | kEntNew (trial state reads it) | kEntOld (accepted state)
};

static_assert(sizeof(FastMove) <= kAuditRecBytes && sizeof(FastMove) % 4 == 0, "audit record size");

// The move after next: its proposal (written by lane 0) and the moved particle's
// resident state, copied from global memory asynchronously one move early.
struct Ahead {
    uint4 rec;
    double x[3];
    double dr[3], u;
    int kind, i, cell;
    float uf;
};

// state only producer lane 0 uses, kept in shared memory so it costs no registers in
// the compute warps (the kernel's register count is the maximum over all threads)
struct ProdState {
    double energy, sum_du; // FP64 folds of accepted energy changes
    FF e_acc;              // accepted finite changes since the last fold
    unsigned long long n_acc, n_mv;
    double M[3];           // sum q r (surface term)
    unsigned long long ctr0;
    long long poff;
    uint32_t sys_id;
    float dp_f;
    long long tprev[2];    // phase timers
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

// A staged proposal (the single-atom fields of fau_proposal).
struct FastProp {
    int kind, index;
    double dr[3];
    double u;
};

// The proposal of move s from the ring into `a` (producer lane 0).  Host proposals are checked
// where they are read: anything but an in-range single-atom move or an empty move (molecular
// moves run in the chain kernel) ends the chain with FAU_ERR_ARG.
__device__ __forceinline__ void fast_proposal(const DevSys& S, const FastProp* ring, long long s, Ahead& a)
{
    const FastProp& f = ring[s % kFastRing];
    const bool ok = f.kind == FAU_MOVE_NONE || (f.kind == FAU_MOVE_ATOMIC && f.index >= 0 && f.index < S.n);
    a.kind = ok ? f.kind : kFastUnsupported;
    a.i = ok ? f.index : 0;
#pragma unroll
    for (int d = 0; d < 3; d++) a.dr[d] = f.dr[d];
    a.u = f.u;
    a.uf = d2f_trunc01(f.u);
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

// Producer lane 0: trial position, record, charge, cells and the layout of the cell
// entries of the move staged in `a`; `prev` is the move evaluated just before it.
// FP64 work per move: the IEEE add and fixed-point rounding of AtomicTranslateRotate's
// new position (3 x add, multiply, convert).
static __device__ __forceinline__ void fast_scalar(const DevSys& S, FastMove& m, const Ahead& a, const FastMove* prev,
                                                const float* itq, const double* itqd, unsigned long long* tsm)
{
    long long t0 = tsm ? clock64() : 0;
    auto sub = [&](int slot) { // profiling only
        if (tsm) {
            const long long now = clock64();
            tsm[slot] += (unsigned long long)(now - t0);
            t0 = now;
        }
    };
    const bool cells = (S.flags & SYS_CELLS) != 0;
    const int kind = a.kind;
    m.kind = kind == kFastUnsupported ? FAU_MOVE_NONE : kind;
    m.i = a.i;
    m.u = a.u;
    m.uf = a.uf;
    m.stop = kind == kFastUnsupported ? FAU_ERR_ARG : 0; // molecular proposal: not handled by this kernel
    m.cap_full = 0;
    m.nue = 0;
    m.conflict = 0;
    if (kind != FAU_MOVE_ATOMIC) {
        m.i = -1;
        m.cell_old = m.cell_new = -1;
        return;
    }
    double xo[3], xn[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        xo[d] = a.x[d];
        xn[d] = __dadd_rn(xo[d], a.dr[d]);
        // Chameleon::boundary only when |x| > L/2 (compared as bit patterns)
        if ((__double_as_longlong(xn[d]) & 0x7FFFFFFFFFFFFFFFLL) > __double_as_longlong(S.half[d]))
            xn[d] = boundary1(xn[d], S.L[d], S.half[d], S.inv[d]);
    }
    const uint4 ro = a.rec;
    const uint4 rn = make_uint4(to_fixed(xn[0], S.fx_scale[0]), to_fixed(xn[1], S.fx_scale[1]),
                                to_fixed(xn[2], S.fx_scale[2]), ro.w);
    sub(20);
    m.ro = ro;
    m.rn = rn;
    m.q = itq[ro.w >> 24];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        m.xo[d] = xo[d];
        m.xn[d] = xn[d];
        // g = dr / L: the proposal's dr equals the minimum-image xn - xo up to the rounding of
        // xo + dr (and whole box lengths, which leave every phase change unchanged); the records'
        // difference would carry their 2^-32 L rounding, too coarse for small moves
        m.g[d] = d2f_trunc(a.dr[d]) * S.inv_f[d];
    }
    if (S.flags & SYS_SURFACE) {
        const double q = itqd[ro.w >> 24];
#pragma unroll
        for (int d = 0; d < 3; d++) m.dM[d] = __dmul_rn(q, __dsub_rn(xn[d], xo[d]));
    }
    if (prev && prev->kind == FAU_MOVE_ATOMIC && prev->i == m.i) m.conflict = FC_SELF;
    sub(22);
    if (cells) {
        const int co = a.cell;
        int c[3], cn[3];
        // the old cell's coordinates: those of the cell the particle is listed in
        if (S.cmag01) {
            const uint32_t c01 = (uint32_t)(S.cdim[0] * S.cdim[1]);
            const uint32_t z = __umulhi((uint32_t)co, S.cmag01), r = (uint32_t)co - z * c01;
            const uint32_t y = __umulhi(r, S.cmag0);
            c[0] = (int)(r - y * (uint32_t)S.cdim[0]);
            c[1] = (int)y;
            c[2] = (int)z;
        }
        else {
            c[0] = co % S.cdim[0];
            c[1] = (co / S.cdim[0]) % S.cdim[1];
            c[2] = co / (S.cdim[0] * S.cdim[1]);
        }
        cell_coords(S, xn, rn, cn);
        m.cell_old = co;
        m.cell_new = cell_index(S, cn);
        bool uni = true;
        int w = 1;
#pragma unroll
        for (int d = 0; d < 3; d++) {
            m.cc_o[d] = c[d];
            m.cc_n[d] = cn[d];
            const int n = S.cdim[d];
            int v = cn[d] - c[d];
            if (2 * v > n) v -= n;
            else if (2 * v < -n) v += n;
            m.df[d] = v;
            if (v < -1 || v > 1 || n < 3 + abs(v)) uni = false;
            m.lo[d] = c[d] + min(v, 0) - 1;
            m.w[d] = 3 + abs(v);
            w *= 3 + abs(v);
        }
        m.uni = uni ? 1 : 0;
        m.nue = uni ? w
                    : 2 * (S.off_max[0] - S.off_min[0] + 1) * (S.off_max[1] - S.off_min[1] + 1) *
                          (S.off_max[2] - S.off_min[2] + 1);
    }
    else {
        m.cell_old = m.cell_new = 0;
    }
    sub(23);
}

// All threads of the CTA but the producer warp (busy committing): the phase tables and the
// cell entries of the move whose scalar part is in `m`.  Dense layout: tables by threads 32,
// 33, ..., entries by threads NT-1, NT-2, ...; SPARSE: entry e by the compute thread that stages
// that cell's records -- thread 32 + e, or with SYS_SPREAD (dense cells) lane e / NWC of compute
// warp e mod NWC, so that every warp holds a share of the stencil -- which also starts the copy
// of the cell's particle count into cnt[e]; the tables from the top.  Returns whether this thread's entries include a cell `prev` (the move
// evaluated just before) rewrote.
template <int MODE>
__device__ __forceinline__ bool fast_parallel(const DevSys& S, FastMove& m, const FastMove& prev, int tid, int NT,
                                              float4* T, int nc, int* cnt)
{
    constexpr bool SPARSE = MODE != 0;
    if (m.kind != FAU_MOVE_ATOMIC) return false;
    const int TS = 2 * nc + 1;
    if (T && tid >= 32) { // per axis and n = -nc..nc: {mid, h}, mid = e^{i n (phi + pi g)}, h = e^{i n pi g}
        for (int e = SPARSE ? NT - 1 - tid : tid - 32; e < 3 * (nc + 1); e += NT - 32) {
            const int ax = e / (nc + 1), n = e - ax * (nc + 1);
            const uint4 ro = m.ro;
            const uint32_t u = ax == 0 ? ro.x : (ax == 1 ? ro.y : ro.z);
            float s, c;
            sincospif((float)n * m.g[ax], &s, &c);
            const float2 mid = cmul(phase_exact((uint32_t)n * u), make_float2(c, s));
            float4* row = T + ax * TS;
            row[nc + n] = make_float4(mid.x, mid.y, c, s);
            row[nc - n] = make_float4(mid.x, -mid.y, c, -s);
        }
    }
    bool hit = false;
    if (S.flags & SYS_CELLS) {
        const int nue = m.nue;
        const int pc_o = prev.kind == FAU_MOVE_ATOMIC ? prev.cell_old : -1;
        const int pc_n = prev.kind == FAU_MOVE_ATOMIC ? prev.cell_new : -1;
        const int nwc = NT / 32 - 1;
        constexpr bool spread = MODE == 2;
        for (int e = SPARSE ? (spread ? ((tid - 32) & 31) * nwc + ((tid - 32) >> 5) : tid - 32) : NT - 1 - tid;
             tid >= 32 && e < nue; e += SPARSE ? 64 : NT - 32) {
            int c[3];
            uint32_t mask;
            if (m.uni) { // one box holding both stencils; each cell flags the states whose stencil contains it
                const int w0 = m.w[0], w1 = m.w[1];
                // box extents are 3 or 4: constant divisors
                const int ex = w0 == 3 ? e % 3 : (e & 3), e1 = w0 == 3 ? e / 3 : (e >> 2);
                const int ey = w1 == 3 ? e1 % 3 : (e1 & 3), ez = w1 == 3 ? e1 / 3 : (e1 >> 2);
                const int o[3] = {m.lo[0] + ex, m.lo[1] + ey, m.lo[2] + ez};
                bool in_o = true, in_n = true;
#pragma unroll
                for (int d = 0; d < 3; d++) {
                    in_o = in_o && abs(o[d] - m.cc_o[d]) <= 1;
                    in_n = in_n && abs(o[d] - (m.cc_o[d] + m.df[d])) <= 1;
                    c[d] = wrap_cell(o[d], S.cdim[d]);
                }
                mask = (in_n ? kEntNew : 0u) | (in_o ? kEntOld : 0u);
            }
            else { // the two neighbour stencils listed separately (GridOffsets3D src/celllistimpl.cpp:15-31)
                const int nbx = S.off_max[0] - S.off_min[0] + 1, nby = S.off_max[1] - S.off_min[1] + 1;
                const int nb = nue / 2;
                const int st = e >= nb ? 1 : 0, r = e - st * nb;
                const int o[3] = {r % nbx + S.off_min[0], (r / nbx) % nby + S.off_min[1], r / (nbx * nby) + S.off_min[2]};
#pragma unroll
                for (int d = 0; d < 3; d++) c[d] = wrap_cell((st ? m.cc_n[d] : m.cc_o[d]) + o[d], S.cdim[d]);
                mask = st ? kEntNew : kEntOld;
            }
            const int cell = cell_index(S, c);
            hit = hit || cell == pc_o || cell == pc_n;
            m.ent[e] = (uint32_t)cell | mask;
            if (SPARSE) { // read again after the barrier when the commit in flight rewrites a cell (hit)
                cp_async(&cnt[e], S.cell_cnt + cell, 4);
                cp_async_commit();
            }
        }
    }
    return hit;
}

struct PairOut {
    float u, mag;
    int flags; // F_* bits of this state
};

// one state of one pair (a single call site keeps the kernel's code small); SPL: the
// instance of splined systems' kernel body (fast_chain_kernel), so that the others keep the
// unsplined register allocation
template <bool SPL>
static __device__ __noinline__ PairOut fast_pair_state(const DevSys& S, PairF p, int pidx, float r2, const double* xi,
                                                        int j, const double* xj, bool is_new)
{
    bool inf = false, nan = false;
    float mag = 0.f;
    const float u = pair_u32<SPL>(S, p, pidx, r2, xi, j, inf, nan, mag, xj);
    PairOut o;
    o.u = u;
    o.mag = mag;
    o.flags = is_new ? ((inf ? F_NEW_INF : 0) | (nan ? F_NEW_NAN : 0)) : ((inf ? F_OLD_INF : 0) | (nan ? F_OLD_NAN : 0));
    return o;
}


// FP64 re-evaluation of move m's energy change (the audit probe): thread ctid of NTC's share --
// its k-vectors and its cell slots (or particles), both states -- as (dU, S) partials, S the
// parity tolerance's error scale (pairs: pair_mag64 in both states; a k-vector:
// A_k (|2 Re(Q* d)| + |d|^2)).  Reciprocal
// space: Q(k) as the chain holds it (FP64 master plus the FP32 pending sums),
// d = q (e^{i k.xn} - e^{i k.xo}) from FP64 phases; pairs: pair_u64 of the FP64 squared distances
// to the resident positions.
__device__ __forceinline__ double2 fast_audit(const DevSys& S, const FastMove& m, int K, int ctid, int NTC, int n_items,
                                              int cap_shift, bool cells)
{
    double du = 0.0, sc = 0.0;
    if (K) {
        const double q = S.itype_qd[m.ro.w >> 24];
        for (int k = ctid; k < K; k += NTC) {
            int nx, ny, nz;
            kn_unpack(S.kn[k], nx, ny, nz);
            // phase / pi = 2 n.x / L
            const double po = 2.0 * ((nx * m.xo[0]) * S.inv[0] + (ny * m.xo[1]) * S.inv[1] + (nz * m.xo[2]) * S.inv[2]);
            const double pn = 2.0 * ((nx * m.xn[0]) * S.inv[0] + (ny * m.xn[1]) * S.inv[1] + (nz * m.xn[2]) * S.inv[2]);
            double so, co, sn, cn;
            sincospi(po, &so, &co);
            sincospi(pn, &sn, &cn);
            const double dx = q * (cn - co), dy = q * (sn - so);
            const double2 qm = S.Q[k];
            const float2 pe = S.qpend[k];
            const double qx = qm.x + (double)pe.x, qy = qm.y + (double)pe.y;
            const double a = S.rec_pref * S.Akd[k];
            const double cross = 2.0 * (qx * dx + qy * dy), dd = dx * dx + dy * dy;
            du += a * (cross + dd);
            sc += a * (fabs(cross) + dd);
        }
    }
    const int ti = (int)(m.rn.w >> 24);
    for (int it = ctid; it < n_items; it += NTC) {
        uint4 rj;
        uint32_t e;
        if (cells) {
            e = m.ent[it >> cap_shift];
            rj = S.cell_rec[(size_t)(e & kEntCell) * S.cap + (it & (S.cap - 1))];
        }
        else {
            e = kEntNew | kEntOld;
            rj = S.rec[it];
        }
        if (rj.w == kEmptySlot) continue;
        const int j = cells ? (int)(rj.w & 0xFFFFFFu) : it;
        if (j == m.i) continue;
        const double xj[3] = {S.x[j], S.y[j], S.z[j]};
        const int tj = (int)(rj.w >> 24);
        if (e & kEntNew) {
            const double r2 = sqdist_d(S, m.xn, xj);
            du += pair_u64(S, ti, tj, r2);
            sc += pair_mag64(S, ti, tj, r2);
        }
        if (e & kEntOld) {
            const double r2 = sqdist_d(S, m.xo, xj);
            du -= pair_u64(S, ti, tj, r2);
            sc += pair_mag64(S, ti, tj, r2);
        }
    }
    return make_double2(du, sc);
}

// Metropolis decision shared by every thread: FP32 unless the exponential is
// within 1e-4 of u (or an infinity, NaN or the surface term is involved), then
// the exact FP64 form metropolisCriterion (src/montecarlo.cpp:17-34) on the
// getEnergyChange value (src/montecarlo.cpp:193-209).  Returns accept; sets
// nan_stop for a NaN energy change.
__device__ __forceinline__ bool fast_decide(FF s, int flags, double du_surf, bool surface, double beta, float beta_f,
                                            double u, float uf, bool& nan_stop)
{
    nan_stop = false;
    if (flags == 0 && !surface) {
        const float xf = (s.hi + s.lo) * beta_f;
        if (xf <= 0.f) return true;
        const float ef = __expf(-xf);
        if (ef > 1e-30f) {
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

// The kernel's static shared memory, declared once in the kernel: the body is inlined twice
// (splined and unsplined systems), and __shared__ variables declared in it would be allocated
// once per inlined copy.
template <int NWC>
struct __align__(16) FastShared {
    DevSys Ssh;             // the system descriptor
    FastMove mvb[3];        // move t, t+1 and the one the producer fills
    Ahead ahs[2];           // move s: ahs[s & 1]
    CommitPre cps[2];       // move s: cps[s & 1]
    FF red_a[2][NWC];
    int red_f[2][NWC];
    float itq[kMaxITypes];
    double itqd[kMaxITypes];
    FastProp ring[kFastRing]; // proposals, filled 32 at a time by the producer warp
    unsigned long long sh_t0; // globaltimer at the start (time-budgeted launches)
    int sh_up;                // the time budget is spent
    int sh_acc;               // the producer's decision of the move: bit 0 accepted, bit 1 NaN stop
    unsigned long long red_u[NWC][2];
    // sparse cell lists: each stencil cell's particle count (per move slot, copied in by the
    // cell's entry thread) and the state flags of each compactly staged record
    int cntb[3][kFastEntries];
    unsigned char sflag[kFastStagePerThread * 32 * NWC];
    // phase timers (profiling only; every phase still runs), accumulated by thread 0 (producer) and
    // thread 32 (first compute warp): 0 commit data, 1 prepare t+1, 2 copies of t+2, 3 barrier 1,
    // 4 decision, 5 commit, 6 conflict barrier | 7 stage, 8 Ewald, 9 pairs, 10 warp sums,
    // 11 barrier 1, 12 decision, 13 Q update, 14 conflict barrier | 15 moves | inside prepare:
    // 16 scalar part, 17 phase tables, 18 cell entries | 21 proposal
    unsigned long long tsm[kFastPhaseSlots];
    ProdState ps;
};

// MODE: 0 whole cells (or all particles); 1 the occupied slots of dilute cells (entries with the
// first warps' lanes, copied cell by cell); 2 the occupied slots of dense cells (entries spread
// over all compute warps, each warp's list copied by all its lanes)
template <int NWC, bool PHILOX, bool SPL, int MODE>
__device__ __forceinline__ void fast_chain_body(const ChainArgs& A, FastShared<NWC>& sh)
{
    constexpr bool SPARSE = MODE != 0;
    constexpr int NT = 32 * (NWC + 1), NTC = 32 * NWC;
    const long long t_start = clock64();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // the system descriptor in shared memory: its fields sit on every move's dependent
    // chain, and global copies fall out of L1 under the cell-list traffic
    DevSys& G = *A.sys[blockIdx.x];
    DevSys& Ssh = sh.Ssh;
    for (int w = tid; w < (int)(sizeof(DevSys) / 8); w += NT)
        reinterpret_cast<unsigned long long*>(&Ssh)[w] = reinterpret_cast<const unsigned long long*>(&G)[w];
    __syncthreads();
    const DevSys& S = Ssh;
    const bool producer = warp == 0;
    const int ctid = tid - 32;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int K = (S.flags & SYS_EWALD) ? S.K : 0;
    const int nc = S.knc;
    const int TS = 2 * nc + 1;
    const int nt = S.nt;
    float4* kq = reinterpret_cast<float4*>(smem_raw); // {Q.x, Q.y, pending.x, pending.y} (FP32 copy + accepted, unflushed)
    float2* dlt = reinterpret_cast<float2*>(kq + K);  // this move's change of Q(k)
    int2* kaf = reinterpret_cast<int2*>(dlt + K);     // {table entries of nx, ny, nz (8 bits each), (2 pi lB / V) A_k}
    float4* tabs = reinterpret_cast<float4*>(kaf + K); // 3 slots x 3 axes x TS phase-table entries {mid, h}
    PairF* pt = reinterpret_cast<PairF*>(tabs + 3 * 3 * TS);
    // pair records (cell slots, or particles without cells) in two half-round buffers, copied in by
    // the compute thread that owns the slot: warp w's items are w's lanes' (no other warp reads them)
    uint4* stage = reinterpret_cast<uint4*>(pt + nt * nt);
    constexpr int KI = kFastStagePerThread / 2, HST = KI * NTC; // records a thread stages and items per half-round
    // SPARSE (MODE 1, 2): only the occupied slots are staged, compactly, each warp in its own
    // region of two buffers of RW records (one round each), from the stencil cells its lanes hold
    constexpr int RW = KI * 32;

    auto& mvb = sh.mvb;
    auto& ahs = sh.ahs;
    auto& cps = sh.cps;
    auto& red_a = sh.red_a;
    auto& red_f = sh.red_f;
    auto& itq = sh.itq;
    auto& itqd = sh.itqd;
    auto& ring = sh.ring;
    auto& sh_t0 = sh.sh_t0;
    auto& sh_up = sh.sh_up;
    auto& red_u = sh.red_u;
    auto& tsm = sh.tsm;
    auto& ps = sh.ps;
    const bool timing = A.phase_cycles != nullptr && (tid == 0 || tid == 32);
    if (tid < kFastPhaseSlots) tsm[tid] = 0;
    auto tick = [&](int slot) {
        if (timing) {
            const long long now = clock64();
            tsm[slot] += (unsigned long long)(now - ps.tprev[tid >> 5]);
            ps.tprev[tid >> 5] = now;
        }
    };

    const float rec_pref_f = (float)S.rec_pref;
    for (int k = tid; k < K; k += NT) {
        const double2 q = S.Q[k];
        const float2 pe = S.qpend[k]; // where the previous launch left the pending changes
        kq[k] = make_float4((float)q.x, (float)q.y, pe.x, pe.y);
        dlt[k] = S.qdlt[k];
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        kaf[k] = make_int2((nx + nc) | ((TS + ny + nc) << 8) | ((2 * TS + nz + nc) << 16),
                           __float_as_int(rec_pref_f * S.Ak[k]));
    }
    for (int t = tid; t < nt * nt; t += NT) pt[t] = S.pair[t];
    if (tid < nt) {
        itq[tid] = S.itype_q[tid];
        itqd[tid] = S.itype_qd[tid];
    }

    const long long nmoves = A.n_moves ? A.n_moves[blockIdx.x] : A.moves;
    // the audit probe: one more move (the chain's next proposal) evaluated after the last one on
    // the final state, never decided or committed; fast_audit_kernel re-evaluates it in FP64
    const long long nloop = nmoves + (A.audit && nmoves > 0 ? 1 : 0);
    if (tid == 0) {
        // cell index -> coordinates by multiply-high: q = umulhi(n, floor((2^32 - 1) / d) + 1) is
        // n / d exactly for n d < 2^32 (n < ncell)
        const unsigned long long d0 = (unsigned long long)Ssh.cdim[0], d01 = d0 * (unsigned long long)Ssh.cdim[1];
        const bool exact = (Ssh.flags & SYS_CELLS) && (unsigned long long)Ssh.ncell * d01 < (1ull << 32);
        Ssh.cmag0 = exact ? (uint32_t)(0xFFFFFFFFull / d0 + 1) : 0u;
        Ssh.cmag01 = exact ? (uint32_t)(0xFFFFFFFFull / d01 + 1) : 0u;
        ps.poff = A.prop_off ? A.prop_off[blockIdx.x] : 0;
        ps.sys_id = A.sys_ids ? A.sys_ids[blockIdx.x] : blockIdx.x;
        ps.ctr0 = A.counters ? A.counters[blockIdx.x] + A.counter_base : A.counter_base;
        ps.dp_f = (float)(A.dp_sys ? A.dp_sys[blockIdx.x] : A.dp);
        ps.energy = S.energy;
        ps.sum_du = 0.0;
        ps.e_acc = FF{S.e_acc_hi, S.e_acc_lo}; // carried over from the previous launch
        ps.n_acc = ps.n_mv = 0;
#pragma unroll
        for (int d = 0; d < 3; d++) ps.M[d] = S.M[d];
        mvb[2].kind = FAU_MOVE_NONE; // "previous move" of move 0
        sh_t0 = global_ns();
        sh_up = 0;
    }
    __syncthreads();
    const bool cells = (S.flags & SYS_CELLS) != 0;
    // SPARSE (the bodies the kernel runs for systems flagged SYS_OCC, which have cells): the
    // occupied slots of the stencil cells only; otherwise whole cells or all particles
    constexpr bool occ = SPARSE;
    const bool surface = (S.flags & SYS_SURFACE) != 0;
    const int cap = S.cap;
    const int cap_shift = cells ? __ffs(cap) - 1 : 0;
    const float beta_f = (float)S.beta_scale;

    // proposals [s0, s0 + 32) into their ring slots, lane w taking move s0 + w: the host's
    // (single-atom fields of fau_proposal), or device proposals drawn here, all 32 at once --
    // philox_proposal's single-atom arithmetic (fau_chain.cuh), so both kernels make the same moves
    auto ring_fill = [&](long long s0) {
        const long long s = s0 + lane;
        if (s >= nloop) return;
        FastProp& f = ring[s % kFastRing];
        if (PHILOX) {
            const Proposal p = philox_proposal(S, ps.ctr0 + (unsigned long long)s, ps.sys_id, A.seed, ps.dp_f, 0.0, false);
            f.kind = p.kind;
            f.index = p.index;
#pragma unroll
            for (int d = 0; d < 3; d++) f.dr[d] = p.dr[d];
            f.u = p.u;
        }
        else { // host streams: the probe repeats the last proposal on the final state
            const fau_proposal& h = A.props[ps.poff + (s < nmoves ? s : nmoves - 1)];
            f.kind = h.kind;
            f.index = h.index;
#pragma unroll
            for (int d = 0; d < 3; d++) f.dr[d] = h.dr[d];
            f.u = h.u;
        }
    };

    unsigned int n_pairs = 0; // this thread's pair evaluations in this launch
    // compute threads: accepts since the FP64 flush; dQ not yet folded in (carried across launches)
    int since_flush = S.q_since, q_pending = S.q_valid;

    // move 0: its scalar part, then tables and cell entries by every thread
    if (producer) {
        ring_fill(0);
        ring_fill(32);
        __syncwarp();
    }
    if (producer && lane == 0 && nmoves > 0) {
        fast_proposal(S, ring, 0, ahs[0]);
        fast_load(S, ahs[0]);
        cp_async_commit();
        cp_async_wait<0>();
        fast_scalar(S, mvb[0], ahs[0], nullptr, itq, itqd, nullptr);
        if (nloop > 1) {
            fast_proposal(S, ring, 1, ahs[1]);
            fast_load(S, ahs[1]);
        }
        fast_commit_loads(S, mvb[0], cps[0]);
        cp_async_commit();
    }
    __syncthreads();
    if (nmoves > 0) fast_parallel<MODE>(S, mvb[0], mvb[2], tid, NT, K ? tabs : nullptr, nc, sh.cntb[0]);
    __syncthreads();

    int prev_accept = 0, stop = 0;
    bool probed = false;
    bool recnt = false;
    if (timing) ps.tprev[tid >> 5] = clock64();
    long long t = 0;
    for (; t < nloop; t++) {
        const int b = (int)(t % 3);
        FastMove& m = mvb[b];
        if (m.stop) {
            stop = m.stop;
            break;
        }
        const int kind = m.kind;
        const int rb = (int)(t & 1);
        if (timing && tid == 0) tsm[15]++;
        if (producer) {
            if ((t & 31) == 0 && t >= 32) {
                ring_fill(t + 32); // proposals [t+32, t+64): first read at move t+30
                __syncwarp();
            }
            if (lane == 0) {
                CommitPre& cp = cps[t & 1];
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
                if (surface && kind == FAU_MOVE_ATOMIC) { // surface-term change of move t (Ewald::updateState)
                    double m2o = 0.0, m2n = 0.0;
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        const double mn = __dadd_rn(ps.M[d], m.dM[d]);
                        m2o = __dadd_rn(m2o, __dmul_rn(ps.M[d], ps.M[d]));
                        m2n = __dadd_rn(m2n, __dmul_rn(mn, mn));
                    }
                    m.du_surf = S.surf_pref * (m2n - m2o);
                }
                tick(0);
                if (t + 1 < nloop) {
                    const FastMove& pm = mvb[(t + 2) % 3]; // move t-1
                    Ahead& an = ahs[(t + 1) & 1];
                    if (t >= 1 && prev_accept && pm.kind == FAU_MOVE_ATOMIC && an.kind == FAU_MOVE_ATOMIC &&
                        an.i == pm.i) { // copied before move t-1's commit: take the committed state
#pragma unroll
                        for (int d = 0; d < 3; d++) an.x[d] = pm.xn[d];
                        an.rec = pm.rn;
                        an.cell = pm.cell_new;
                    }
                    fast_scalar(S, mvb[(t + 1) % 3], an, &m, itq, itqd, timing ? tsm : nullptr);
                    tick(1);
                    if (t + 2 < nloop) {
                        Ahead& a2 = ahs[t & 1];
                        fast_proposal(S, ring, t + 2, a2);
                        tick(21);
                        fast_load(S, a2);
                    }
                    fast_commit_loads(S, mvb[(t + 1) % 3], cps[(t + 1) & 1]);
                }
                cp_async_commit(); // group 2: Ahead of move t+2, commit counts of move t+1
                tick(2);
            }
        }
        else if (kind == FAU_MOVE_ATOMIC) {
            const int i = m.i;
            const uint4 ro = m.ro, rn = m.rn;
            const int ti = rn.w >> 24;
            const int n_items = cells ? (m.nue << cap_shift) : S.n;
            auto item_src = [&](int it) -> const uint4* {
                return cells ? S.cell_rec + (size_t)(m.ent[it >> cap_shift] & kEntCell) * cap + (it & (cap - 1))
                             : S.rec + it;
            };
            // this thread's records of half-round h (items [h HST, (h + 1) HST)): asynchronous copies
            // into buffer h & 1, one commit group a half-round
            auto stage_half = [&](int h) {
                uint4* buf = stage + (h & 1) * HST;
#pragma unroll
                for (int k = 0; k < KI; k++) {
                    const int it = h * HST + ctid + k * NTC;
                    if (it < n_items) cp_async(&buf[ctid + k * NTC], item_src(it), 16);
                }
                cp_async_commit();
            };
            // SPARSE: this lane's stencil cell (entry my_e), its particle count (read again now
            // when the last commit rewrote a cell of the stencil), and the records' place in the
            // warp's compact list: an exclusive prefix over the warp's lanes.  The list is copied
            // by all lanes, RW records a round into one of two buffers of the warp's region
            const int my_e = MODE == 2 ? lane * NWC + (warp - 1) : ctid;
            const int n_ent = my_e < m.nue ? 1 : 0;
            const int w_ent = __popc(__ballot_sync(0xffffffffu, n_ent)); // entries of this warp: lanes 0..
            uint4* buf_w = stage + (warp - 1) * 2 * RW;
            unsigned char* fl_w = sh.sflag + (warp - 1) * 2 * RW;
            uint32_t my_ent = 0;
            int my_cnt = 0, my_off = 0, w_total = 0;
            bool per_cell = MODE == 1; // cell by cell (dilute cells); 2: by all lanes of the warp
            auto stage_sparse = [&](int h) { // records [h RW, (h + 1) RW) of the warp's list
                uint4* dst = buf_w + (h & 1) * RW;
                unsigned char* fd = fl_w + (h & 1) * RW;
                if (MODE == 1 || per_cell) {
                    const uint4* src = S.cell_rec + (size_t)(my_ent & kEntCell) * cap;
                    const unsigned char f = (unsigned char)(my_ent >> 30);
                    for (int j = 0; j < my_cnt; j++) {
                        const int c = my_off + j - h * RW;
                        if (c >= 0 && c < RW) {
                            cp_async(&dst[c], src + j, 16);
                            fd[c] = f;
                        }
                    }
                    cp_async_commit();
                    return;
                }
#pragma unroll
                for (int k = 0; k < KI; k++) {
                    const int c = h * RW + lane + 32 * k;
                    // the entry holding record c: the last of the warp's entries starting at or before it
                    int lo = 0;
#pragma unroll
                    for (int step = 16; step > 0; step >>= 1) {
                        const int mid = lo + step;
                        const int om = __shfl_sync(0xffffffffu, my_off, mid & 31);
                        if (mid < w_ent && om <= c) lo = mid;
                    }
                    const uint32_t ent = __shfl_sync(0xffffffffu, my_ent, lo);
                    const int oo = __shfl_sync(0xffffffffu, my_off, lo);
                    if (c < w_total) {
                        cp_async(&dst[lane + 32 * k], S.cell_rec + (size_t)(ent & kEntCell) * cap + (c - oo), 16);
                        fd[lane + 32 * k] = (unsigned char)(ent >> 30);
                    }
                }
                cp_async_commit();
            };
            int n_half = 0;
            // SPARSE: started part-way through the Ewald loop, when the counts copied in during the
            // last move have landed; the records then land during the rest of it
            auto stage_sparse0 = [&]() {
                if (n_ent) {
                    int* cnt = sh.cntb[b];
                    my_ent = m.ent[my_e];
                    if (recnt) {
                        cp_async_wait<0>(); // the earlier copy lands first
                        cp_async(&cnt[my_e], S.cell_cnt + (my_ent & kEntCell), 4);
                        cp_async_commit();
                    }
                    cp_async_wait<0>();
                    my_cnt = min(max(cnt[my_e], 0), cap);
                }
                int incl = my_cnt;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int v = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += v;
                }
                my_off = incl - my_cnt;
                w_total = __shfl_sync(0xffffffffu, incl, 31);
                if constexpr (MODE == 2) per_cell = __reduce_max_sync(0xffffffffu, (unsigned)my_cnt) <= 4u;
                n_half = (w_total + RW - 1) / RW; // rounds of RW records
                if (n_half > 0) stage_sparse(0);
                if (n_half > 1) stage_sparse(1);
            };
            if constexpr (!occ) {
                n_half = (n_items + HST - 1) / HST;
                stage_half(0); // the first two half-rounds land while the Ewald loop runs
                if (n_half > 1) stage_half(1);
            }
            tick(7);
            // ---- Ewald: one k-vector per thread and step, two independent accumulators.  The
            // last accepted move's Q(k) change (State::sync trial -> accepted) is folded in here,
            // in the same pass; every 256 accepts the FP32 pending sums go to the FP64 master.
            FF acc0{0.f, 0.f}, acc1{0.f, 0.f};
            if (K) {
                if (q_pending && since_flush >= kFastFlushAccepts) {
                    for (int k = ctid; k < K; k += NTC) {
                        const float4 qq = kq[k];
                        const float2 d = dlt[k];
                        double2 q = S.Q[k];
                        q.x += (double)(qq.z + d.x);
                        q.y += (double)(qq.w + d.y);
                        S.Q[k] = q;
                        kq[k] = make_float4((float)q.x, (float)q.y, 0.f, 0.f);
                    }
                    q_pending = 0;
                    since_flush = 0;
                }
                const bool pa = q_pending != 0;
                const float4* Tb = tabs + b * 3 * TS;
                const float f0 = 2.f * m.q;
                // (2 pi lB / V) A_k (|Q + d|^2 - |Q|^2) for one k-vector; dQ(k) = d kept for the commit
                auto ewald_k = [&](int k) {
                    float4 qq = kq[k];
                    if (pa) {
                        const float2 dp = dlt[k];
                        qq.z += dp.x;
                        qq.w += dp.y;
                        kq[k] = qq;
                    }
                    const int2 ka = kaf[k];
                    const float4 tx = Tb[ka.x & 0xff], ty = Tb[(ka.x >> 8) & 0xff], tz = Tb[ka.x >> 16];
                    const float2 mid = cmul(cmul(make_float2(tx.x, tx.y), make_float2(ty.x, ty.y)), make_float2(tz.x, tz.y));
                    const float2 hxy = cmul(make_float2(tx.z, tx.w), make_float2(ty.z, ty.w));
                    const float f = f0 * fmaf(hxy.x, tz.w, hxy.y * tz.z); // 2 q sin(D/2)
                    dlt[k] = make_float2(-f * mid.y, f * mid.x);             // d = 2 q sin(D/2) i mid
                    const float qx = qq.x + qq.z, qy = qq.y + qq.w;
                    // 2 Re(Q* d) + |d|^2 = f (2 (Qy mid.x - Qx mid.y) + f)
                    const float r = fmaf(qy, mid.x, -qx * mid.y);
                    return __int_as_float(ka.y) * (f * fmaf(2.f, r, f));
                };
                int k = ctid;
                if constexpr (SPARSE) {
                    for (int it = 0; it < 2 && k + NTC < K; it++, k += 2 * NTC) {
                        const float ta = ewald_k(k), tb = ewald_k(k + NTC);
                        ff_add(acc0, ta + tb);
                    }
                    stage_sparse0();
                }
                for (; k + NTC < K; k += 2 * NTC) {
                    const float ta = ewald_k(k), tb = ewald_k(k + NTC);
                    ff_add(acc0, ta + tb);
                }
                if (k < K) ff_add(acc1, ewald_k(k));
                q_pending = 0;
            }
            else if constexpr (occ) {
                stage_sparse0();
            }
            FF accp = ff_sum(acc0, acc1);
            int flags = 0;
            tick(8);

            // ---- pairs: the staged records of a round.  A (record, state) pair is a task when the slot
            // is occupied by another particle, the state's stencil holds its cell, and the state's
            // FP32 r^2 lies below the pair cutoff with twice the FP64 guard band: beyond it every term
            // is exactly 0 with no flag (pair_u32), so leaving it out changes no sum.  The tasks are
            // counted per warp and each lane evaluates one, reading its record from the stage, so a
            // round costs one pass per 32 tasks
            const unsigned FULL = 0xffffffffu;
            const int wbase = (warp - 1) * 32;
            const float cut2 = S.rc2_pair > 0.f ? S.rc2_pair * 1.00002f : __int_as_float(0x7f800000);
            for (int h = 0; occ && h < n_half; h++) {
                // round h of the warp's compact list: every record is an occupied slot of a stencil
                // cell, with that cell's state flags (bit 0 trial state, bit 1 accepted state)
                if (h + 1 < n_half) cp_async_wait<1>(); // round h landed (h + 1 may still be in flight)
                else cp_async_wait<0>();
                __syncwarp();
                const uint4* bw = buf_w + (h & 1) * RW;
                const unsigned char* fw = fl_w + (h & 1) * RW;
                const int nrec = min(RW, w_total - h * RW);
                unsigned occ[2 * KI];
                int nv = 0;
#pragma unroll
                for (int k = 0; k < KI; k++) {
                    const int it = lane + 32 * k;
                    bool on = false, oo = false;
                    if (it < nrec) {
                        const uint4 r = bw[it];
                        const uint32_t f = fw[it];
                        if (r.w != kEmptySlot && (int)(r.w & 0xFFFFFFu) != i) {
                            on = (f & 1u) && r2_fixed(S, rn, r) < cut2;
                            oo = (f & 2u) && r2_fixed(S, ro, r) < cut2;
                        }
                    }
                    occ[2 * k] = __ballot_sync(FULL, on);
                    occ[2 * k + 1] = __ballot_sync(FULL, oo);
                    nv += __popc(occ[2 * k]) + __popc(occ[2 * k + 1]);
                }
                for (int base = 0; base < nv; base += 32) {
                    const int q = base + lane;
                    if (q < nv) {
                        int qq = q, mi = 0;
                        unsigned mk = occ[0];
#pragma unroll
                        for (int kk = 1; kk < 2 * KI; kk++) {
                            const int c = __popc(mk);
                            if (mi == kk - 1 && qq >= c) {
                                qq -= c;
                                mi = kk;
                                mk = occ[kk];
                            }
                        }
                        const int src = (int)__fns(mk, 0, qq + 1);
                        const int st = mi & 1;
                        const uint4 rj = bw[src + (mi >> 1) * 32];
                        const int j = (int)(rj.w & 0xFFFFFFu);
                        const int pidx = ti * nt + (int)(rj.w >> 24);
                        const PairOut o = fast_pair_state<SPL>(S, pt[pidx], pidx, r2_fixed(S, st ? ro : rn, rj),
                                                               st ? m.xo : m.xn, j, nullptr, st == 0);
                        ff_add(accp, st ? -o.u : o.u);
                        flags |= o.flags;
                        if (t < nmoves) n_pairs++;
                    }
                }
                if (h + 2 < n_half) { // refill this buffer with round h + 2
                    __syncwarp(); // every lane done reading it
                    stage_sparse(h + 2);
                }
            }
            for (int h = 0; !occ && h < n_half; h++) {
                // half-round h complete (h + 1, when there is one, may still be in flight)
                if (h + 1 < n_half) cp_async_wait<1>();
                else cp_async_wait<0>();
                __syncwarp(); // every lane's copies visible to the warp
                const uint4* buf = stage + (h & 1) * HST;
                const int r0 = h * HST;
                unsigned occ[2 * KI]; // per staged record k: [2k] trial state, [2k + 1] accepted state
                int nv = 0;
#pragma unroll
                for (int k = 0; k < KI; k++) {
                    const int it = r0 + ctid + k * NTC;
                    bool on = false, oo = false;
                    if (it < n_items) {
                        const uint4 r = buf[ctid + k * NTC];
                        const uint32_t e = cells ? m.ent[it >> cap_shift] : (kEntNew | kEntOld);
                        if (r.w != kEmptySlot && (cells ? (int)(r.w & 0xFFFFFFu) : it) != i) {
                            on = (e & kEntNew) && r2_fixed(S, rn, r) < cut2;
                            oo = (e & kEntOld) && r2_fixed(S, ro, r) < cut2;
                        }
                    }
                    occ[2 * k] = __ballot_sync(FULL, on);
                    occ[2 * k + 1] = __ballot_sync(FULL, oo);
                    nv += __popc(occ[2 * k]) + __popc(occ[2 * k + 1]);
                }
                for (int base = 0; base < nv; base += 32) {
                    const int q = base + lane;
                    if (q < nv) {
                        // the q-th task of this warp's half-round: its mask and rank in it
                        int qq = q, mi = 0;
                        unsigned mk = occ[0];
#pragma unroll
                        for (int kk = 1; kk < 2 * KI; kk++) {
                            const int c = __popc(mk);
                            if (mi == kk - 1 && qq >= c) {
                                qq -= c;
                                mi = kk;
                                mk = occ[kk];
                            }
                        }
                        const int src = (int)__fns(mk, 0, qq + 1);
                        const int st = mi & 1; // 1: the accepted state
                        const int slot = wbase + src + (mi >> 1) * NTC;
                        const uint4 rj = buf[slot];
                        const int j = cells ? (int)(rj.w & 0xFFFFFFu) : r0 + slot;
                        const int pidx = ti * nt + (int)(rj.w >> 24);
                        const PairOut o = fast_pair_state<SPL>(S, pt[pidx], pidx, r2_fixed(S, st ? ro : rn, rj),
                                                               st ? m.xo : m.xn, j, nullptr, st == 0);
                        ff_add(accp, st ? -o.u : o.u);
                        flags |= o.flags;
                        if (t < nmoves) n_pairs++; // not the audit probe's
                    }
                }
                if (h + 2 < n_half) { // refill this buffer with half-round h + 2
                    __syncwarp(); // every lane done reading it
                    stage_half(h + 2);
                }
            }
            tick(9);
            float sc_unused = 0.f;
            FF b_unused{0.f, 0.f};
            warp_reduce(accp, b_unused, sc_unused, flags, false);
            if (lane == 0) {
                red_a[rb][warp - 1] = accp;
                red_f[rb][warp - 1] = flags;
            }
            tick(10);
        }
        __syncthreads(); // B0
        tick(tid == 0 ? 3 : 11);
        if (t == nmoves) { // the audit probe: evaluated only
            probed = true;
            break;
        }

        // ---- decision by the producer warp (the warp partials summed as a tree, the same order
        // in every lane); the compute warps go on to the next move and read it after B1
        int accept = 0;
        bool nan_stop = false;
        if (producer) {
            double du_surf = 0.0;
            FF s{0.f, 0.f};
            int fl = 0;
            if (kind == FAU_MOVE_ATOMIC) {
                FF part[NWC];
#pragma unroll
                for (int w = 0; w < NWC; w++) {
                    part[w] = red_a[rb][w];
                    fl |= red_f[rb][w];
                }
#pragma unroll
                for (int h = 1; h < NWC; h <<= 1)
#pragma unroll
                    for (int w = 0; w + h < NWC; w += 2 * h) part[w] = ff_sum(part[w], part[w + h]);
                s = part[0];
                if (surface) du_surf = m.du_surf;
                accept = fast_decide(s, fl, du_surf, surface, S.beta_scale, beta_f, m.u, m.uf, nan_stop) ? 1 : 0;
            }
            if (nan_stop) accept = 0;
            tick(4);
            if (lane == 0 && !nan_stop) {
                FF dff{0.f, 0.f}; // this move's energy change as float-float (written packed to du_out)
                if (kind == FAU_MOVE_ATOMIC) {
                    ps.n_mv++;
                    if (fl == 0 && !surface) {
                        dff = s;
                        if (accept) {
                            ps.n_acc++;
                            ps.e_acc = ff_sum(ps.e_acc, s);
                        }
                    }
                    else if (accept || A.du_out) {
                        const double du = energy_change(ff_value(s) + du_surf, fl & F_NEW_INF, fl & F_OLD_INF,
                                                        fl & F_NEW_NAN, fl & F_OLD_NAN);
                        dff.hi = (float)du;
                        dff.lo = isfinite(du) ? (float)(du - (double)dff.hi) : 0.f;
                        if (accept) {
                            ps.n_acc++;
                            const double acc = ff_value(ps.e_acc);
                            ps.energy += acc + du;
                            ps.sum_du += acc + du;
                            ps.e_acc = FF{0.f, 0.f};
                        }
                    }
                }
                const long long po = ps.poff + t;
                if (A.acc_out) A.acc_out[po] = (uint8_t)accept;
                if (A.du_out) // packed {hi, lo}; a kernel after the launch turns the range into doubles
                    reinterpret_cast<float2*>(A.du_out)[po] = make_float2(dff.hi, dff.lo);
                if (accept && surface) {
#pragma unroll
                    for (int d = 0; d < 3; d++) ps.M[d] = __dadd_rn(ps.M[d], m.dM[d]);
                }
                if (accept) { // commit (State::sync trial -> accepted): positions, record, cell list
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
                        G.err = FAU_ERR_STATE; // inconsistent cell list: leave it untouched
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
                tick(5);
            }
            if (lane == 0) sh.sh_acc = accept | (nan_stop ? 2 : 0);
        }
        // ---- the next move: re-prepared (after a barrier) if it moves the particle of this
        // move and this move was accepted, then its phase tables and cell entries by every thread
        bool hit = false;
        if (t + 1 < nloop) {
            FastMove& nm = mvb[(t + 1) % 3];
            if (nm.conflict & FC_SELF) {
                if (producer && lane == 0 && accept) {
                    Ahead& an = ahs[(t + 1) & 1];
                    cp_async_wait<0>();
                    fast_proposal(S, ring, t + 1, an);
                    fast_load(S, an);
                    cp_async_commit();
                    cp_async_wait<0>();
                    fast_scalar(S, nm, an, &m, itq, itqd, nullptr);
                    fast_commit_loads(S, nm, cps[(t + 1) & 1]);
                    cp_async_commit();
                }
                __syncthreads();
            }
            hit = fast_parallel<MODE>(S, nm, m, tid, NT, K ? tabs + ((t + 1) % 3) * 3 * TS : nullptr, nc,
                                        sh.cntb[(t + 1) % 3]);
        }
        tick(tid == 0 ? 6 : 13);
        if (A.time_budget_ns && tid == 0 && global_ns() - sh_t0 >= A.time_budget_ns) sh_up = 1;
        hit = __syncthreads_or(hit) != 0; // B1: decision, commit, tables and entries visible
        recnt = hit; // SPARSE: the next move's counts of cells this commit rewrote are read again
        if (hit && producer && lane == 0) mvb[(t + 1) % 3].conflict |= FC_CELLS;
        tick(tid == 0 ? 6 : 14);
        {
            const int af = sh.sh_acc;
            accept = af & 1;
            if (af & 2) { // a NaN energy change: the launch ends before this move
                stop = FAU_ERR_NAN;
                break;
            }
        }
        if (accept) {
            if (!producer && K) { // this thread's share of Q(k) += dQ(k), folded into the next Ewald pass
                q_pending = 1;
                since_flush++;
            }
            if (m.cap_full) { // committed; the launch ends after it
                stop = FAU_ERR_CAPACITY;
                break;
            }
        }
        prev_accept = accept;
        if (sh_up && t + 1 < nmoves) { // the time budget is spent: the launch ends after move t (after
            t++;                        // the last move it still runs the audit probe)
            break;
        }
    }
    cp_async_wait<0>(); // no copy outlives the CTA (the producer's loads, sparse cell counts)
    __syncthreads();
    // the audit probe's record: its FP32 energy change (the warp partials the loop left before B0)
    // and the move itself, for fast_audit_kernel after this launch
    if (probed && G.audit_rec) {
        const FastMove& pm = mvb[t % 3];
        const int words = (int)(sizeof(FastMove) / 4);
        for (int w = tid; w < words; w += NT)
            reinterpret_cast<uint32_t*>(G.audit_rec)[w] = reinterpret_cast<const uint32_t*>(&pm)[w];
        if (tid == 0) {
            FF s32{0.f, 0.f};
            int fl = 0;
            for (int w = 0; w < NWC; w++) {
                s32 = ff_sum(s32, red_a[t & 1][w]);
                fl |= red_f[t & 1][w];
            }
            G.audit_du = ff_value(s32) + (surface && pm.kind == FAU_MOVE_ATOMIC ? pm.du_surf : 0.0);
            G.audit_pending = pm.kind == FAU_MOVE_ATOMIC && fl == 0 ? 1 : 0; // finite in both states
        }
    }
    if (A.phase_cycles && tid < kFastPhaseSlots && tsm[tid])
        atomicAdd(&A.phase_cycles[blockIdx.x * kFastPhaseSlots + tid], tsm[tid]);

    // the pending changes stay pending: the next launch continues from them exactly as the next
    // move would (the host folds them into the master before it reads Q)
    if (!producer) {
        for (int k = ctid; k < K; k += NTC) {
            const float4 qq = kq[k];
            S.qpend[k] = make_float2(qq.z, qq.w);
            S.qdlt[k] = dlt[k];
        }
        if (ctid == 0) {
            G.q_valid = K ? q_pending : 0;
            G.q_since = K ? since_flush : 0;
        }
    }
    unsigned long long pa = n_pairs;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) pa += __shfl_xor_sync(0xffffffffu, pa, o);
    if (!producer && lane == 0) red_u[warp - 1][0] = pa;
    __syncthreads();
    if (tid == 0) {
        unsigned long long sp = 0;
        for (int w = 0; w < NWC; w++) sp += red_u[w][0];
        G.pair_evals += sp;
        G.k_updates += ps.n_mv * (unsigned long long)K; // every k-vector once per single-atom move
        // the float-float part stays unfolded for the next launch; sum_du counts it once
        const double acc = ff_value(ps.e_acc), acc0 = (double)S.e_acc_hi + (double)S.e_acc_lo;
        G.moves += ps.n_mv;
        G.accepted += ps.n_acc;
        G.sum_du += ps.sum_du + (acc - acc0);
        G.energy = ps.energy;
        G.e_acc_hi = ps.e_acc.hi;
        G.e_acc_lo = ps.e_acc.lo;
#pragma unroll
        for (int d = 0; d < 3; d++) G.M[d] = ps.M[d];
        if (stop) G.err = stop;
        G.consumed = stop == FAU_ERR_CAPACITY ? t + 1 : t;
        G.cycles += (unsigned long long)(clock64() - t_start);
    }
}

// The body up to four times, selected per CTA by its system: splined systems (FAU_PAIR_SPLINE)
// get their own instance, so the pair path of the others compiles exactly as without the tables,
// and the three staging modes each theirs.
template <int NWC, bool PHILOX, bool SPARSE>
__global__ void __launch_bounds__(32 * (NWC + 1), NWC <= 2 ? 6 : (NWC <= 4 ? 4 : 2)) fast_chain_kernel(ChainArgs A)
{
    __shared__ FastShared<NWC> sh;
    // SPARSE instances: systems flagged SYS_OCC (fast_occupied_slots; cell lists) run the body
    // that stages the occupied slots of stencil cells, the others the whole-cell body; splined
    // systems their own.  The choice depends only on the system.
    const DevSys* G = A.sys[blockIdx.x];
    const bool occ = SPARSE && (G->flags & SYS_OCC) && (G->flags & SYS_CELLS);
    if (G->terms & FAU_PAIR_SPLINE) fast_chain_body<NWC, PHILOX, true, 0>(A, sh);
    else if (occ && (G->flags & SYS_SPREAD)) fast_chain_body<NWC, PHILOX, false, SPARSE ? 2 : 0>(A, sh);
    else if (occ) fast_chain_body<NWC, PHILOX, false, SPARSE ? 1 : 0>(A, sh);
    else fast_chain_body<NWC, PHILOX, false, 0>(A, sh);
}

// dynamic shared memory of the pipelined kernel for K k-vectors, table size nc, nt classes and
// NWC compute warps (their staged pair records come last)
__host__ __device__ inline size_t fast_smem_bytes(int K, int nc, int nt, int nwc)
{
    return (size_t)K * (sizeof(float4) + sizeof(float2) + sizeof(int2)) + (size_t)3 * 3 * (2 * nc + 1) * sizeof(float4) +
           (size_t)nt * nt * sizeof(PairF) + (size_t)fast_stage_items(nwc) * sizeof(uint4);
}

template <int NWC, bool PH, bool SPARSE = false>
cudaError_t launch_fast_inst(const ChainArgs& a, int nblocks, int K, int nc, int nt, cudaStream_t st, bool prepare_only)
{
    // the dynamic allowance is raised on demand, never inside a stream capture: callers prepare first
    static size_t granted = 0;
    const size_t smem = fast_smem_bytes(K, nc, nt, NWC);
    if (smem > granted || granted == 0) {
        cudaError_t e = cudaFuncSetAttribute(fast_chain_kernel<NWC, PH, SPARSE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        granted = smem;
    }
    if (prepare_only) return cudaSuccess;
    fast_chain_kernel<NWC, PH, SPARSE><<<nblocks, 32 * (NWC + 1), smem, st>>>(a);
    return cudaGetLastError();
}

} // namespace fau
