// fau_chain.cuh -- the persistent Metropolis chain kernel (one CTA per chain).
//
// One loop iteration is one MetropolisMonteCarlo::performMove
// (reference src/montecarlo.cpp:139-187) for a transrot or moltransrot move:
//
//   [all warps]  apply the previous move's Q(k) change if it was accepted,
//                then evaluate this move: Ewald dU over the CTA's k-vectors
//                (two-per-axis phase tables, see below) and the pair dU over
//                the cell-list neighbours (or all particles), accumulated in
//                float-float per thread and per warp
//   barrier
//   [warp 0]     final sum, getEnergyChange + metropolisCriterion (FP64),
//                commit positions / records / cell list / mass centre,
//                prepare the next move (FP64 trial positions, phase tables)
//   barrier
//
// Ewald phases: for a moved atom with fixed-point position u and
// displacement g = (r_new - r_old) / L (minimum image), the CTA builds per
// axis the tables e^{i n 2 pi u_d / 2^32} and e^{i n pi g_d} for n = -nc..nc
// (sincospi of exactly reduced integer phases, 6 (2 nc + 1) entries).  Every
// k-vector then needs five complex products:
//     e_old = ex[nx] ey[ny] ez[nz],   h = e^{i D/2} = hx[nx] hy[ny] hz[nz],
//     d     = q (e_new - e_old) = 2 q sin(D/2) i e_old h,
// which keeps d accurate for small moves (no e_new - e_old cancellation).
#pragma once
#include "fau_dev.cuh"
#include "fau_kernels.h"

namespace fau {

constexpr int kTableAtoms = 8; // moved atoms handled with phase tables (larger groups: direct sincospi)
constexpr int kNblChunk = 512;  // candidate groups per GroupCutoff pass of a molecular move (multiple of NT)
constexpr uint32_t kNblNew = 1u << 30, kNblOld = 1u << 31, kNblGroup = kNblNew - 1u;

struct MoveShared {
    int kind, index, m, first;
    int accept, stop, prev_accept, pad;
    long long consumed;
    double u;
    int cc_old[3], cc_new[3]; // cell coordinates of the moved atom (atomic moves with cells)
    int cell_old, cell_new;
    float q[kMaxGroupAtoms];
    float3 g[kMaxGroupAtoms]; // minimum-image displacement / L per moved atom
    uint4 rec_old[kMaxGroupAtoms];
    uint4 rec_new[kMaxGroupAtoms];
    double xn[kMaxGroupAtoms][3];
    double xo[kMaxGroupAtoms][3];
    double cm_new[3];
    double dM[3];
    uint4 cmrec_old, cmrec_new;
};

// cell coordinates of a position: fixed-point fast path; the FP64 reference formula
// floor((x + L/2) / cell_len) (src/celllistimpl.h:139-143, src/sasa.cpp:466-468)
// decides within 2^-18 of a cell boundary, so binning is bit-exact.
// one axis d: x the FP64 coordinate, u its fixed-point record
__device__ __forceinline__ int cell_coord1(const DevSys& S, double x, uint32_t u, int d)
{
    const uint32_t s = u + 0x80000000u;
    const unsigned long long prod = (unsigned long long)s * (unsigned long long)S.cdim[d];
    int v = (int)(prod >> 32);
    const uint32_t frac = (uint32_t)prod;
    if (frac < (1u << 14) || frac > 0xFFFFFFFFu - (1u << 14)) {
        const double t = __dadd_rn(x, __dmul_rn(0.5, S.L[d]));
        v = (int)floor(__ddiv_rn(t, S.cell_len[d]));
    }
    if (v < 0) v += S.cdim[d] * (abs(v) / S.cdim[d] + 1);
    else if (v >= S.cdim[d]) v -= S.cdim[d] * (v / S.cdim[d]);
    return v;
}
__device__ __forceinline__ void cell_coords(const DevSys& S, const double* x, uint4 r, int* c)
{
    const uint32_t u[3] = {r.x, r.y, r.z};
#pragma unroll
    for (int d = 0; d < 3; d++) c[d] = cell_coord1(S, x[d], u[d], d);
}
__device__ __forceinline__ int cell_index(const DevSys& S, const int* c)
{
    return c[0] + S.cdim[0] * (c[1] + S.cdim[1] * c[2]);
}

// GroupCutoff::cut (src/energy.h:761-768): sqdist(cm1, cm2) >= cutoff^2, FP32 on
// fixed-point mass centres, FP64 inside a 1e-5 guard band.  c2 < 0: no cutoff.
__device__ __forceinline__ bool group_cut_rec(const DevSys& S, uint4 cmrec, const double* cm, uint4 cmrec_h, int h,
                                              double c2, float c2f)
{
    if (c2 < 0.0) return false;
    const float r2 = r2_fixed(S, cmrec, cmrec_h);
    if (r2 < c2f * 0.99999f) return false;
    if (r2 > c2f * 1.00001f) return true;
    const double o[3] = {S.g_cm[3 * h], S.g_cm[3 * h + 1], S.g_cm[3 * h + 2]};
    return sqdist_d(S, cm, o) >= c2;
}

// quaternion rotation v' = v + w t + u x t, t = 2 u x v (FP64, never contracted)
// The neighbour-group list of a molecular move: warp v lists its GroupCutoff survivors in its
// own segment [v * seg, v * seg + wc[v]) in (row, lane) order. The list order, and with it the
// order of every pair sum, is then independent of the order in which warps arrive, so dU is
// reproducible bit for bit. Slot of the q-th listed group:
template <int NWL>
__device__ __forceinline__ int nbl_slot(int q, const int (&wc)[NWL], int seg)
{
    int off = 0;
    bool found = false;
#pragma unroll
    for (int v = 0; v < NWL; v++) {
        if (!found && q >= wc[v]) {
            q -= wc[v];
            off += seg;
        }
        else {
            found = true;
        }
    }
    return off + q;
}

__device__ __forceinline__ void quat_rotate(const double* q, double* v)
{
    const double ux = q[1], uy = q[2], uz = q[3], w = q[0];
    double tx = __dsub_rn(__dmul_rn(uy, v[2]), __dmul_rn(uz, v[1]));
    double ty = __dsub_rn(__dmul_rn(uz, v[0]), __dmul_rn(ux, v[2]));
    double tz = __dsub_rn(__dmul_rn(ux, v[1]), __dmul_rn(uy, v[0]));
    tx = __dadd_rn(tx, tx);
    ty = __dadd_rn(ty, ty);
    tz = __dadd_rn(tz, tz);
    const double cx = __dsub_rn(__dmul_rn(uy, tz), __dmul_rn(uz, ty));
    const double cy = __dsub_rn(__dmul_rn(uz, tx), __dmul_rn(ux, tz));
    const double cz = __dsub_rn(__dmul_rn(ux, ty), __dmul_rn(uy, tx));
    v[0] = __dadd_rn(__dadd_rn(v[0], __dmul_rn(w, tx)), cx);
    v[1] = __dadd_rn(__dadd_rn(v[1], __dmul_rn(w, ty)), cy);
    v[2] = __dadd_rn(__dadd_rn(v[2], __dmul_rn(w, tz)), cz);
}

struct Proposal {
    int kind, index;
    double dr[3];
    double quat[4];
    double u;
    float uf; // u truncated to float (decides unless within 1e-4 of the threshold)
    bool rotate;
};

// Device-RNG proposal (batched mode), a deliberate deviation from the reference's
// mt19937 stream: uniform direction (Archimedes), |dr| = dp U(0,1) computed in FP32
// and widened exactly, uniform particle / group, 53-bit Metropolis uniform.  The
// doubles are assembled from bit patterns (no FP64 instruction on this path).
static __device__ __noinline__ Proposal philox_proposal(const DevSys& S, unsigned long long ctr, uint32_t sys_id, uint64_t seed,
                                           float dp, double dprot, bool molecular)
{
    Proposal p;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const U4 c1 = philox({(uint32_t)ctr, (uint32_t)(ctr >> 32), sys_id, 0u}, k0, k1);
    const U4 c2 = philox({(uint32_t)ctr, (uint32_t)(ctr >> 32), sys_id, 1u}, k0, k1);
    const float z = fmaf(2.f, u01_24(c1.y), -1.f);
    float s, c;
    sincospif(2.f * u01_24(c1.z), &s, &c);
    const float rxy = sqrtf(fmaxf(0.f, 1.f - z * z));
    const float len = dp * u01_24(c1.w);
    p.dr[0] = f2d_bits(rxy * c * len);
    p.dr[1] = f2d_bits(rxy * s * len);
    p.dr[2] = f2d_bits(z * len);
    const unsigned long long v = ((unsigned long long)(c2.x >> 5) << 26) | (c2.y >> 6);
    p.u = u53_bits(v);
    // u truncated to float (relative error below 2^-23, as for host proposals): an absolute 2^-24
    // grid would let the FP32 prefilter misjudge u within 2^-24 of a threshold below 6e-4
    p.uf = d2f_trunc01(p.u);
    p.rotate = false;
    p.quat[0] = 1.0;
    p.quat[1] = p.quat[2] = p.quat[3] = 0.0;
    if (!molecular) {
        // no displacement is an empty Change, as AtomicTranslateRotate::_move makes it (src/move.cpp:267-293)
        p.kind = dp > 0.f ? FAU_MOVE_ATOMIC : FAU_MOVE_NONE;
        const uint32_t n = S.n_atomic > 0 ? (uint32_t)S.n_atomic : (uint32_t)S.n;
        const uint32_t j = __umulhi(c1.x, n);
        p.index = S.n_atomic > 0 ? S.atomic_idx[j] : (int)j;
    }
    else {
        // no translation and no rotation is an empty Change (TranslateRotate::_move, src/move.cpp:1670-1689)
        p.kind = (dp > 0.f || dprot > 0.0) ? FAU_MOVE_MOLECULAR : FAU_MOVE_NONE;
        p.index = (int)__umulhi(c1.x, (uint32_t)S.n_groups);
        if (dprot > 0.0) {
            // uniform axis, angle dprot (U - 1/2); the half-angle sine/cosine and the axis come
            // from the FP32 pipe (FP64 sin/cos is ~100 instructions on a slow pipe) and the
            // quaternion (cos, sin a) is normalised once in FP64, so rotations stay unit to FP64
            // precision.  The FP32 axis' norm (1 within 2^-22) scales tan(angle / 2) by the same
            // factor whatever the sign of the angle, so the proposal stays symmetric.
            const float az = fmaf(2.f, u01_24(c2.z), -1.f);
            float as, ac;
            sincospif(2.f * u01_24(c2.w), &as, &ac);
            const float axy = sqrtf(fmaxf(0.f, 1.f - az * az));
            const U4 c3 = philox({(uint32_t)ctr, (uint32_t)(ctr >> 32), sys_id, 2u}, k0, k1);
            const float ha_pi = (float)dprot * (u01_24(c3.x) - 0.5f) * (0.5f / 3.14159265358979f); // angle / (2 pi)
            float sh, ch;
            sincospif(ha_pi, &sh, &ch);
            const double ax = f2d_bits(axy * ac), ay = f2d_bits(axy * as), az_d = f2d_bits(az);
            const double c = f2d_bits(ch), s = f2d_bits(sh);
            const double q0 = c, q1 = s * ax, q2 = s * ay, q3 = s * az_d;
            const double rq = rsqrt(q0 * q0 + q1 * q1 + q2 * q2 + q3 * q3);
            p.quat[0] = q0 * rq;
            p.quat[1] = q1 * rq;
            p.quat[2] = q2 * rq;
            p.quat[3] = q3 * rq;
            p.rotate = true;
        }
    }
    return p;
}

__device__ __forceinline__ Proposal load_proposal(const fau_proposal& f)
{
    Proposal p;
    p.kind = f.kind;
    p.index = f.index;
#pragma unroll
    for (int d = 0; d < 3; d++) p.dr[d] = f.dr[d];
#pragma unroll
    for (int d = 0; d < 4; d++) p.quat[d] = f.quat[d];
    p.u = f.u;
    p.uf = d2f_trunc01(f.u);
    p.rotate = !(f.quat[0] == 0.0 && f.quat[1] == 0.0 && f.quat[2] == 0.0 && f.quat[3] == 0.0);
    return p;
}

// (xn - xo) / L of axis d under minimum image; |v| > L/2 compared as bit patterns
__device__ __forceinline__ float min_image_frac1(const DevSys& S, double xn, double xo, int d)
{
    double v = __dsub_rn(xn, xo);
    const long long b = __double_as_longlong(v);
    if ((b & 0x7FFFFFFFFFFFFFFFLL) > __double_as_longlong(S.half[d])) v = b < 0 ? __dadd_rn(v, S.L[d]) : __dsub_rn(v, S.L[d]);
    return (float)v * S.inv_f[d];
}

// (xn - xo) / L per axis under minimum image (Chameleon::vdist src/geometry.h:429-458)
__device__ __forceinline__ float3 min_image_frac(const DevSys& S, const double* xn, const double* xo)
{
    return make_float3(min_image_frac1(S, xn[0], xo[0], 0), min_image_frac1(S, xn[1], xo[1], 1),
                       min_image_frac1(S, xn[2], xo[2], 2));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}

// e^{i pi P 2^-31} for an exact 32-bit phase P: sincospi of the top 24 bits
// (exact in FP32) times the first-order rotation by the remaining 8 bits.
__device__ __forceinline__ float2 phase_exact(uint32_t P)
{
    const uint32_t hi = P & 0xFFFFFF00u;
    const float th = (float)(int32_t)hi * 4.656612873077393e-10f;          // 2^-31
    const float dl = (float)(P & 0xFFu) * (3.14159265358979f * 4.656612873077393e-10f);
    float s, c;
    sincospif(th, &s, &c);
    return make_float2(fmaf(-s, dl, c), fmaf(c, dl, s));
}

// Warp 0: proposal -> FP64 trial positions (AtomicTranslateRotate::translateParticle
// src/move.cpp:225-240; Group::translate src/group.cpp:115-123 then Group::rotate
// src/group.cpp:110-113, src/geometry.h:613-627), fixed-point records, cells, and
// the phase tables of the moved atoms.
static __device__ __noinline__ void prepare_move(const DevSys& S, MoveShared& ms, const Proposal& p, int lane, float2* tab, int nc,
                                                 unsigned long long* tsub = nullptr)
{
    const long long tp0 = tsub ? clock64() : 0;
    const int TS = 2 * nc + 1;
    // host proposals are checked here, where they are read: an index out of range or an unknown
    // kind ends the chain with FAU_ERR_ARG before anything is indexed with it
    const bool bad = p.kind == FAU_MOVE_ATOMIC ? (p.index < 0 || p.index >= S.n)
                     : p.kind == FAU_MOVE_MOLECULAR ? (p.index < 0 || p.index >= S.n_groups)
                                                    : p.kind != FAU_MOVE_NONE;
    if (bad) {
        if (lane == 0) {
            ms.kind = FAU_MOVE_NONE;
            ms.index = -1;
            ms.m = 0;
            ms.first = -1;
            ms.stop = FAU_ERR_ARG;
        }
        __syncwarp();
        return;
    }
    if (lane == 0) {
        ms.kind = p.kind;
        ms.index = p.index;
        ms.u = p.u;
        ms.stop = 0;
    }
    int m = 0;
    if (p.kind == FAU_MOVE_ATOMIC) {
        m = 1;
        if (lane == 0) {
            const int i = p.index;
            const double xo[3] = {S.x[i], S.y[i], S.z[i]};
            double xn[3];
#pragma unroll
            for (int d = 0; d < 3; d++) xn[d] = boundary1(__dadd_rn(xo[d], p.dr[d]), S.L[d], S.half[d], S.inv[d]);
            const uint4 ro = S.rec[i];
            uint4 rn;
            rn.x = to_fixed(xn[0], S.fx_scale[0]);
            rn.y = to_fixed(xn[1], S.fx_scale[1]);
            rn.z = to_fixed(xn[2], S.fx_scale[2]);
            rn.w = ro.w;
            ms.m = 1;
            ms.first = i;
            ms.rec_old[0] = ro;
            ms.rec_new[0] = rn;
            const double q = S.itype_qd[ro.w >> 24];
            ms.q[0] = (float)q;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                ms.xn[0][d] = xn[d];
                ms.xo[0][d] = xo[d];
                ms.dM[d] = __dmul_rn(q, __dsub_rn(xn[d], xo[d]));
            }
            ms.g[0] = min_image_frac(S, xn, xo);
            if (S.flags & SYS_CELLS) {
                const int co = S.cell_of[i];
                ms.cell_old = co;
                ms.cc_old[0] = co % S.cdim[0];
                ms.cc_old[1] = (co / S.cdim[0]) % S.cdim[1];
                ms.cc_old[2] = co / (S.cdim[0] * S.cdim[1]);
                int c[3];
                cell_coords(S, xn, rn, c);
                ms.cc_new[0] = c[0];
                ms.cc_new[1] = c[1];
                ms.cc_new[2] = c[2];
                ms.cell_new = cell_index(S, c);
            }
        }
    }
    else if (p.kind == FAU_MOVE_MOLECULAR) {
        // One lane per (atom, axis), ten atoms a round: the FP64 pipe issues one warp instruction
        // per 64 cycles whatever the number of active lanes, so the three coordinates' chains
        // share each instruction.  Every lane runs the same operations on the same values as a
        // per-atom evaluation (Group::translate, Group::rotate, geometry.h:613-627), so the
        // positions are the same bits; the rotation's cross products take the other two
        // coordinates from the atom's other lanes.
        const int g = p.index;
        const int b = S.g_begin[g];
        m = S.g_begin[g + 1] - b;
        const unsigned FULL = 0xffffffffu;
        const int dl = lane % 3, la = lane / 3, lb = lane - dl;
        const int l1 = lb + (dl + 1) % 3, l2 = lb + (dl + 2) % 3; // lanes of axes d+1, d+2 (mod 3)
        const double Ld = S.L[dl], hd = S.half[dl], id = S.inv[dl];
        const double cmd = boundary1(__dadd_rn(S.g_cm[3 * g + dl], p.dr[dl]), Ld, hd, id);
        const double u1 = p.quat[1 + (dl + 1) % 3], u2 = p.quat[1 + (dl + 2) % 3];
        const double* X = dl == 0 ? S.x : (dl == 1 ? S.y : S.z);
        double dMs = 0.0; // lanes 0..2: the group's dipole change, summed in atom order
        for (int a0 = 0; m <= kMaxGroupAtoms && a0 < m; a0 += 10) { // uniform over the warp
            const int a = a0 + la;
            const bool act = lane < 30 && a < m;
            const int i = b + (act ? a : 0);
            const double xo = X[i];
            double v = boundary1(__dadd_rn(xo, p.dr[dl]), Ld, hd, id);
            if (p.rotate) {
                v = boundary1(__dsub_rn(v, cmd), Ld, hd, id);
                const double v1 = __shfl_sync(FULL, v, l1), v2 = __shfl_sync(FULL, v, l2);
                double t = __dsub_rn(__dmul_rn(u1, v2), __dmul_rn(u2, v1)); // t = 2 u x v
                t = __dadd_rn(t, t);
                const double t1 = __shfl_sync(FULL, t, l1), t2 = __shfl_sync(FULL, t, l2);
                const double c = __dsub_rn(__dmul_rn(u1, t2), __dmul_rn(u2, t1)); // u x t
                v = __dadd_rn(__dadd_rn(v, __dmul_rn(p.quat[0], t)), c);
                v = boundary1(__dadd_rn(v, cmd), Ld, hd, id);
            }
            const uint4 ro = S.rec[i];
            const double q = S.itype_qd[ro.w >> 24];
            const double dMa = __dmul_rn(q, __dsub_rn(v, xo));
            if (act) {
                reinterpret_cast<uint32_t*>(&ms.rec_new[a])[dl] = to_fixed(v, S.fx_scale[dl]);
                ms.xn[a][dl] = v;
                ms.xo[a][dl] = xo;
                reinterpret_cast<float*>(&ms.g[a])[dl] = min_image_frac1(S, v, xo, dl);
                if (dl == 0) {
                    ms.rec_old[a] = ro;
                    ms.rec_new[a].w = ro.w;
                    ms.q[a] = (float)q;
                }
            }
            const int na = min(10, m - a0);
            for (int k = 0; k < na; k++) { // lane d adds atom a0 + k's component d
                const double x = __shfl_sync(FULL, dMa, 3 * k + dl);
                if (lane < 3) dMs = __dadd_rn(dMs, x);
            }
        }
        if (lane < 3) {
            ms.cm_new[dl] = cmd;
            ms.dM[dl] = dMs;
            reinterpret_cast<uint32_t*>(&ms.cmrec_new)[dl] = to_fixed(cmd, S.fx_scale[dl]);
        }
        if (lane == 0) {
            ms.m = m;
            ms.first = b;
            if (m > kMaxGroupAtoms) ms.stop = FAU_ERR_ARG;
            ms.cmrec_old = S.g_cmrec[g];
            ms.cmrec_new.w = 0u;
        }
    }
    else if (lane == 0) {
        ms.m = 0;
        ms.first = -1;
    }
    __syncwarp();
    const long long tp1 = tsub ? clock64() : 0;
    // phase tables: per atom (a < min(m, kTableAtoms)), per axis d, n = 0..nc
    if (tab && m <= kTableAtoms) {
        const int per_atom = 6 * (nc + 1);
        for (int e = lane; e < m * per_atom; e += 32) {
            const int a = e / per_atom, r = e - a * per_atom;
            const int kind = r / (nc + 1), n = r - kind * (nc + 1); // kind 0..2: old phase, 3..5: half delta
            float2 v;
            if (kind < 3) {
                const uint4 ro = ms.rec_old[a];
                const uint32_t u = kind == 0 ? ro.x : (kind == 1 ? ro.y : ro.z);
                v = phase_exact((uint32_t)n * u);
            }
            else {
                const float3 g = ms.g[a];
                const float gd = kind == 3 ? g.x : (kind == 4 ? g.y : g.z);
                float s, c;
                sincospif((float)n * gd, &s, &c);
                v = make_float2(c, s);
            }
            float2* t = tab + (a * 6 + kind) * TS;
            t[nc + n] = v;
            t[nc - n] = make_float2(v.x, -v.y);
        }
    }
    if (tsub) { // profiling: positions, then phase tables
        const long long tp2 = clock64();
        tsub[0] += (unsigned long long)(tp1 - tp0);
        tsub[1] += (unsigned long long)(tp2 - tp1);
    }
}

// metropolisCriterion (src/montecarlo.cpp:17-34) for a non-NaN du: FP32 exp decides
// unless u is within 1e-4 of the threshold; then the FP64 u <= exp(-du) decides.
__device__ __forceinline__ bool metropolis(double du, double u)
{
    if (isinf(du) && du < 0.0) return true;
    if (-du > 709.782712893384) return true;
    if (du <= 0.0 && u < 1.0) return true; // exp(-du) >= 1 > u
    const float ef = __expf((float)(-du));
    if (ef > 1e-30f) {
        if (u < (double)ef * 0.9999) return true;
        if (u > (double)ef * 1.0001) return false;
    }
    else if (u > 1e-29) {
        return false;
    }
    return u <= exp(-du);
}

// getEnergyChange (src/montecarlo.cpp:193-209) from per-state inf/NaN flags
__device__ __forceinline__ double energy_change(double finite_du, bool new_inf, bool old_inf, bool new_nan,
                                                bool old_nan)
{
    const double inf = __longlong_as_double(0x7ff0000000000000ULL);
    if (old_nan && !new_nan) return -inf;
    if (new_nan) return inf;
    if (new_inf) return inf;
    if (old_inf) return -inf;
    return finite_du;
}

enum : int { F_NEW_INF = 1, F_OLD_INF = 2, F_NEW_NAN = 4, F_OLD_NAN = 8 };

__device__ __forceinline__ void add_pair(FF& acc, int& flags, float un, float uo, bool ni, bool oi, bool nn, bool on)
{
    ff_add(acc, un - uo);
    flags |= (ni ? F_NEW_INF : 0) | (oi ? F_OLD_INF : 0) | (nn ? F_NEW_NAN : 0) | (on ? F_OLD_NAN : 0);
}

__device__ __forceinline__ void warp_reduce(FF& a, FF& b, float& sc, int& flags, bool two)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF ta{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
        a = ff_sum(a, ta);
        if (two) {
            FF tb{__shfl_xor_sync(0xffffffffu, b.hi, o), __shfl_xor_sync(0xffffffffu, b.lo, o)};
            b = ff_sum(b, tb);
            sc += __shfl_xor_sync(0xffffffffu, sc, o);
        }
    }
    flags = __reduce_or_sync(0xffffffffu, flags);
}

// at most 128 registers a thread: two 256-thread (four 128-thread) systems per SM
template <int NT, bool PHILOX>
__global__ void __launch_bounds__(NT, 65536 / (NT * 128)) chain_kernel(ChainArgs A)
{
    constexpr int NW = NT / 32;
    const long long t_start = clock64();
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // the system descriptor in shared memory: its fields sit on every move's dependent
    // chain, and global copies fall out of L1 under the cell-list traffic
    DevSys& G = *A.sys[blockIdx.x];
    __shared__ __align__(16) DevSys Ssh;
    for (int w = tid; w < (int)(sizeof(DevSys) / 8); w += NT)
        reinterpret_cast<unsigned long long*>(&Ssh)[w] = reinterpret_cast<const unsigned long long*>(&G)[w];
    __syncthreads();
    const DevSys& S = Ssh;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int K = (S.flags & SYS_EWALD) ? S.K : 0;
    const int nc = S.knc;
    const int TS = 2 * nc + 1;
    float2* Qb = reinterpret_cast<float2*>(smem_raw); // FP32 copy of the FP64 master Q
    float2* pend = Qb + K;                            // accepted changes not yet flushed to FP64
    float2* dlt = pend + K;                           // this move's change of Q(k)
    int* kidx = reinterpret_cast<int*>(dlt + K);      // table indices (nx+nc) | (ny+nc)<<8 | (nz+nc)<<16
    float* Af = reinterpret_cast<float*>(kidx + K);   // (2 pi lB / V) A_k
    float2* tab = reinterpret_cast<float2*>(Af + K);  // kTableAtoms * 6 * TS phase tables

    __shared__ PairF pt[kMaxITypes * kMaxITypes];
    __shared__ MoveShared ms;
    __shared__ FF red_a[NW], red_b[NW];
    __shared__ float red_s[NW];
    __shared__ int red_f[NW];
    // a finite maxenergy: the trial state's Nonbonded sum and the accepted state's reciprocal
    // energy, reduced beside the energy change
    __shared__ FF red_n[NW], red_o[NW];
    __shared__ int nbo[27][3];
    __shared__ uint32_t nbl[kNblChunk]; // molecular moves: neighbour groups of one chunk | interacting states
    __shared__ int nbl_wcnt[NW];        // survivors each warp listed in its segment

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
    int nnb = 0, gshift = 0;
    if (S.flags & SYS_CELLS) {
        const int nbx = S.off_max[0] - S.off_min[0] + 1, nby = S.off_max[1] - S.off_min[1] + 1,
                  nbz = S.off_max[2] - S.off_min[2] + 1;
        nnb = nbx * nby * nbz;
        if (tid < nnb) {
            nbo[tid][0] = tid % nbx + S.off_min[0];
            nbo[tid][1] = (tid / nbx) % nby + S.off_min[1];
            nbo[tid][2] = tid / (nbx * nby) + S.off_min[2];
        }
        while ((2 * nnb) << (gshift + 1) <= NT) gshift++; // G = 2^gshift lanes per (state, cell)
    }

    const long long nmoves = A.n_moves ? A.n_moves[blockIdx.x] : A.moves;
    const long long poff = A.prop_off ? A.prop_off[blockIdx.x] : 0;
    const uint32_t sys_id = A.sys_ids ? A.sys_ids[blockIdx.x] : blockIdx.x;
    const unsigned long long ctr0 = A.counters ? A.counters[blockIdx.x] + A.counter_base : A.counter_base;
    const bool molecular_sys = A.molecular ? (A.molecular[blockIdx.x] != 0) : false;
    const float dp_f = (float)(A.dp_sys ? A.dp_sys[blockIdx.x] : A.dp);
    const double dprot = A.dprot_sys ? A.dprot_sys[blockIdx.x] : A.dprot;
    const bool detail = A.detail != nullptr;
    const int nt = S.nt;
    // the audit probe (batched and stream launches; not the evaluate-only mode or a finite
    // maxenergy): one more move, the chain's next proposal (a host stream's last one again),
    // evaluated after the last one on the final state and never decided or committed; its FP32
    // energy change and the move go to the system's audit record for probe_audit_kernel
    const long long nloop = nmoves + (A.audit && nmoves > 0 && !A.pending && !S.maxe && G.audit_rec ? 1 : 0);

    unsigned long long n_acc = 0, n_pairs = 0, n_k = 0, n_mv = 0;
    int since_flush = S.q_since;
    double energy = sys_energy(S), sum_du = 0.0; // the pipelined kernel's unfolded part folded in
    double M[3] = {S.M[0], S.M[1], S.M[2]};

    // phase timers (profiling only; every phase still runs): slots
    // 0 deferred Q commit, 1 Ewald, 2 pairs, 3 reduce + barrier 1, 4 decision, 5 commit,
    // 6 prepare next, 7 barrier 2 (warp 0); 8 compute, 9 barrier 1, 10 barrier 2 (warp 1); last: moves
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
    __shared__ unsigned long long sh_t0; // globaltimer at the start (time-budgeted launches)
    __shared__ long long sh_up_at;       // >= 0: the time budget ended the launch after this many moves
    if (tid == 0) {
        ms.prev_accept = S.q_valid; // the previous launch's last accepted change, if not yet folded
        ms.consumed = 0;
        sh_t0 = global_ns();
        sh_up_at = -1;
    }
    __syncthreads();
    if (warp == 0 && nmoves > 0) {
        const Proposal p = PHILOX ? philox_proposal(S, ctr0, sys_id, A.seed, dp_f, dprot, molecular_sys)
                                  : load_proposal(A.props[poff]);
        prepare_move(S, ms, p, lane, K ? tab : nullptr, nc);
    }
    __syncthreads();

    for (long long mv = 0; mv < nloop; mv++) {
        const bool probe = mv == nmoves; // after the last move the audit probe runs, time budget or not
        if (ms.stop || (sh_up_at >= 0 && !probe)) break;
        const unsigned long long n_pairs0 = n_pairs, n_k0 = n_k; // the probe's evaluations are not counted
        // ---- the previous move's Q(k) change (State::sync trial -> accepted, deferred)
        if (ms.prev_accept) {
            for (int k = tid; k < K; k += NT) {
                float2 pe = pend[k];
                const float2 d = dlt[k];
                pe.x += d.x;
                pe.y += d.y;
                pend[k] = pe;
            }
            if (++since_flush == kFlushAccepts) { // FP32 pending -> FP64 master
                since_flush = 0;
                for (int k = tid; k < K; k += NT) {
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
        const int kind = ms.kind;
        const int m = ms.m;
        if (timing) {
            tick(0);
            if (tid == 0) tacc[kPhaseSlots - 1]++;
        }

        // ---- energy change of this move
        FF accp{0.f, 0.f}, accr{0.f, 0.f};
        FF accn{0.f, 0.f}, acco{0.f, 0.f}; // maxenergy: sum u(trial state), sum A_k |Q_k|^2 (accepted)
        const bool maxe = S.maxe != 0;
        float scale = 0.f;
        int flags = 0;
        if (kind != FAU_MOVE_NONE) {
            if (K) {
                // one thread per k-vector (strided): d = sum_a q_a (e_new - e_old) from the phase tables
                if (m == 1) {
                    const float2* t = tab;
                    const float f0 = 2.f * ms.q[0];
                    for (int k = tid; k < K; k += NT) {
                        const int ki = kidx[k];
                        const int ix = ki & 0xff, iy = (ki >> 8) & 0xff, iz = ki >> 16;
                        const float2 qb = Qb[k], pe = pend[k];
                        const float af = Af[k];
                        const float2 eo = cmul(t[ix], cmul(t[TS + iy], t[2 * TS + iz]));
                        const float2 h = cmul(t[3 * TS + ix], cmul(t[4 * TS + iy], t[5 * TS + iz]));
                        const float2 pp = cmul(eo, h);
                        const float f = f0 * h.y;
                        const float2 d = make_float2(-f * pp.y, f * pp.x);
                        dlt[k] = d;
                        const float qx = qb.x + pe.x, qy = qb.y + pe.y;
                        const float cross = 2.f * fmaf(qx, d.x, qy * d.y);
                        const float dd = fmaf(d.x, d.x, d.y * d.y);
                        ff_add(accr, af * (cross + dd));
                        if (detail) scale += af * (fabsf(cross) + dd);
                        if (maxe) ff_add(acco, af * fmaf(qx, qx, qy * qy));
                    }
                }
                else {
                    const bool tables = m <= kTableAtoms;
                    for (int k = tid; k < K; k += NT) {
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
                            else { // large groups: direct phases
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
                        const float af = Af[k];
                        ff_add(accr, af * (cross + dd));
                        if (detail) scale += af * (fabsf(cross) + dd);
                        if (maxe) ff_add(acco, af * fmaf(qx, qx, qy * qy));
                    }
                }
                n_k += (unsigned long long)m * (unsigned long long)((K - tid + NT - 1) / NT > 0 ? (K - tid + NT - 1) / NT : 0);
                if (A.pending_dq)
                    for (int k = tid; k < K; k += NT) A.pending_dq[k] = make_double2((double)dlt[k].x, (double)dlt[k].y);
            }
            tick(tid == 0 ? 1 : 8);

            if (kind == FAU_MOVE_ATOMIC) {
                const int i = ms.index;
                const uint4 rn = ms.rec_new[0], ro = ms.rec_old[0];
                const int ti = rn.w >> 24;
                if (S.flags & SYS_CELLS) {
                    const int G = 1 << gshift;
                    const int items = (2 * nnb) << gshift;
                    for (int it = tid; it < items; it += NT) {
                        const int sc = it >> gshift, sub = it & (G - 1);
                        const int state = sc >= nnb ? 1 : 0;
                        const int c = sc - state * nnb;
                        const int* cc = state ? ms.cc_new : ms.cc_old;
                        int v[3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            int w = cc[d] + nbo[c][d];
                            if (w < 0) w += S.cdim[d];
                            else if (w >= S.cdim[d]) w -= S.cdim[d];
                            v[d] = w;
                        }
                        const int cell = v[0] + S.cdim[0] * (v[1] + S.cdim[1] * v[2]);
                        const int cnt = S.cell_cnt[cell];
                        const uint4* cr = S.cell_rec + (size_t)cell * S.cap;
                        const uint4 ri = state ? rn : ro;
                        const double* xi = state ? ms.xn[0] : ms.xo[0];
                        for (int s = sub; s < cnt; s += G) {
                            const uint4 rj = cr[s];
                            const int j = (int)(rj.w & 0xFFFFFFu);
                            if (j == i) continue;
                            const int pidx = ti * nt + (rj.w >> 24);
                            bool inf = false, nan = false;
                            float mg = 0.f;
                            const float u = pair_u32(S, pt[pidx], pidx, r2_fixed(S, ri, rj), xi, j, inf, nan, mg);
                            if (state) {
                                add_pair(accp, flags, u, 0.f, inf, false, nan, false);
                                if (maxe) ff_add(accn, u);
                            }
                            else {
                                add_pair(accp, flags, 0.f, u, false, inf, false, nan);
                            }
                            if (detail) scale += mg;
                            n_pairs++;
                        }
                    }
                }
                else {
                    for (int j = tid; j < S.n; j += NT) {
                        if (j == i) continue;
                        const uint4 rj = S.rec[j];
                        const int pidx = ti * nt + (rj.w >> 24);
                        const PairF p = pt[pidx];
                        float uu[2];
                        bool fi[2], fn[2];
                        float mg = 0.f;
                        for (int st = 0; st < 2; st++) { // st 0: trial (new), 1: accepted (old)
                            fi[st] = false;
                            fn[st] = false;
                            uu[st] = pair_u32(S, p, pidx, r2_fixed(S, st ? ro : rn, rj), st ? ms.xo[0] : ms.xn[0], j,
                                              fi[st], fn[st], mg);
                        }
                        add_pair(accp, flags, uu[0], uu[1], fi[0], fi[1], fn[0], fn[1]);
                        if (maxe) ff_add(accn, uu[0]);
                        if (detail) scale += mg;
                        n_pairs += 2;
                    }
                }
            }
            else if (kind == FAU_MOVE_MOLECULAR) { // group2all(group) with GroupCutoff
                const int g = ms.index;
                const uint4 cmo = ms.cmrec_old, cmn = ms.cmrec_new;
                const double cmo_d[3] = {S.g_cm[3 * g], S.g_cm[3 * g + 1], S.g_cm[3 * g + 2]};
                // In chunks of kNblChunk candidate groups: (1) the GroupCutoff tests, survivors
                // compacted into `nbl` with the states they interact in; (2) one (neighbour
                // group, moved atom) task per thread over the list -- every thread does
                // useful pair work instead of a few lanes running whole groups serially.
                const int G = S.n_groups;
                const int mol_g = S.n_mol > 0 ? S.g_molid[g] : 0;
                for (int base = 0; base < G; base += kNblChunk) {
                    constexpr int RC = kNblChunk / NT;
                    constexpr int SEG = RC * 32; // each warp tests RC * 32 candidates per chunk
                    int wc = 0;
                    int gfl[RC], gml[RC];
                    uint4 gcr[RC];
#pragma unroll
                    for (int r = 0; r < RC; r++) { // all loads first: their latencies overlap
                        const int h = base + r * NT + tid;
                        gfl[r] = h < G ? S.g_flags[h] : FAU_GROUP_ATOMIC;
                        gcr[r] = h < G ? S.g_cmrec[h] : make_uint4(0, 0, 0, 0);
                        gml[r] = (h < G && S.n_mol > 0) ? S.g_molid[h] : 0;
                    }
#pragma unroll
                    for (int r = 0; r < RC; r++) {
                        const int h = base + r * NT + tid;
                        uint32_t e = 0;
                        if (h < G && h != g && !(gfl[r] & FAU_GROUP_ATOMIC)) {
                            double c2 = S.cut_g2g2;
                            float c2f = S.cut_g2g2f;
                            if (S.n_mol > 0) { // GroupCutoff::getCutoff(molid of g, molid of h)
                                const int k = mol_g * S.n_mol + gml[r];
                                c2 = S.cut2_mol[k];
                                c2f = S.cut2_molf[k];
                            }
                            const bool cut_o = group_cut_rec(S, cmo, cmo_d, gcr[r], h, c2, c2f);
                            const bool cut_n = group_cut_rec(S, cmn, ms.cm_new, gcr[r], h, c2, c2f);
                            e = (cut_n ? 0u : kNblNew) | (cut_o ? 0u : kNblOld);
                        }
                        const unsigned bal = __ballot_sync(0xffffffffu, e != 0);
                        if (e) nbl[warp * SEG + wc + __popc(bal & ((1u << lane) - 1u))] = (uint32_t)h | e;
                        wc += __popc(bal);
                    }
                    if (lane == 0) nbl_wcnt[warp] = wc;
                    __syncthreads();
                    int wcl[NW], cnt = 0;
#pragma unroll
                    for (int v = 0; v < NW; v++) {
                        wcl[v] = nbl_wcnt[v];
                        cnt += wcl[v];
                    }
                    for (int task = tid; task < cnt * m; task += NT) {
                        const int q = task / m, a = task - q * m;
                        const uint32_t ent = nbl[nbl_slot(q, wcl, SEG)];
                        const int h = (int)(ent & kNblGroup);
                        const bool do_n = (ent & kNblNew) != 0, do_o = (ent & kNblOld) != 0;
                        const int hb = S.g_begin[h], he = S.g_begin[h + 1];
                        const uint4 ra_n = ms.rec_new[a], ra_o = ms.rec_old[a];
                        const int ta = ra_n.w >> 24;
                        for (int b = hb; b < he; b++) {
                            const uint4 rb = S.rec[b];
                            const int pidx = ta * nt + (int)(rb.w >> 24);
                            const PairF p = pt[pidx];
                            float uu[2] = {0.f, 0.f};
                            bool fi[2] = {false, false}, fn[2] = {false, false};
                            float mg = 0.f;
                            for (int st = 0; st < 2; st++) {
                                if (!(st ? do_o : do_n)) continue;
                                uu[st] = pair_u32(S, p, pidx, r2_fixed(S, st ? ra_o : ra_n, rb), st ? ms.xo[a] : ms.xn[a],
                                                  b, fi[st], fn[st], mg);
                                n_pairs++;
                            }
                            add_pair(accp, flags, uu[0], uu[1], fi[0], fi[1], fn[0], fn[1]);
                            if (maxe) ff_add(accn, uu[0]);
                            if (detail) scale += mg;
                        }
                    }
                    __syncthreads();
                }
                for (int t = tid; t < S.n_atomic; t += NT) { // atomic groups are never cut
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
                        if (maxe) ff_add(accn, uu[0]);
                        if (detail) scale += mg;
                        n_pairs += 2;
                    }
                }
            }
        }

        tick(tid == 0 ? 2 : 8);
        // ---- reduce: per warp, then warp 0 (B1)
        const bool sep = detail || maxe; // the pair and reciprocal parts kept apart
        if (!sep) accp = ff_sum(accp, accr);
        warp_reduce(accp, accr, scale, flags, sep);
        if (maxe) {
            float sc_n = 0.f;
            int fl_n = 0;
            warp_reduce(accn, acco, sc_n, fl_n, true);
        }
        if (lane == 0) {
            red_a[warp] = accp;
            red_b[warp] = accr;
            red_s[warp] = scale;
            red_f[warp] = flags;
            if (maxe) {
                red_n[warp] = accn;
                red_o[warp] = acco;
            }
        }
        __syncthreads();
        tick(tid == 0 ? 3 : 9);
        if (probe) {
            n_pairs = n_pairs0;
            n_k = n_k0;
            if (warp == 0) {
                accp = lane < NW ? red_a[lane] : FF{0.f, 0.f};
                accr = lane < NW ? red_b[lane] : FF{0.f, 0.f};
                flags = lane < NW ? red_f[lane] : 0;
#pragma unroll
                for (int o = NW / 2; o > 0; o >>= 1) {
                    FF ta{__shfl_xor_sync(0xffffffffu, accp.hi, o), __shfl_xor_sync(0xffffffffu, accp.lo, o)};
                    accp = ff_sum(accp, ta);
                    if (sep) {
                        FF tb{__shfl_xor_sync(0xffffffffu, accr.hi, o), __shfl_xor_sync(0xffffffffu, accr.lo, o)};
                        accr = ff_sum(accr, tb);
                    }
                    flags |= __shfl_xor_sync(0xffffffffu, flags, o);
                }
                ProbeRecord& pr = *reinterpret_cast<ProbeRecord*>(G.audit_rec);
                const int mm = kind == FAU_MOVE_NONE ? 0 : m;
                if (lane < mm) {
#pragma unroll
                    for (int d = 0; d < 3; d++) pr.xn[lane][d] = ms.xn[lane][d];
                }
                if (lane == 0) {
                    double du_surf = 0.0;
                    if (kind != FAU_MOVE_NONE && (S.flags & SYS_SURFACE)) {
                        double m2o = 0.0, m2n = 0.0;
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            const double mn = __dadd_rn(M[d], ms.dM[d]);
                            m2o = __dadd_rn(m2o, __dmul_rn(M[d], M[d]));
                            m2n = __dadd_rn(m2n, __dmul_rn(mn, mn));
                        }
                        du_surf = S.surf_pref * (m2n - m2o);
                    }
                    pr.kind = kind;
                    pr.index = ms.index;
                    pr.m = mm;
                    pr.first = ms.first;
#pragma unroll
                    for (int d = 0; d < 3; d++) {
                        pr.cm_new[d] = ms.cm_new[d];
                        pr.dM[d] = ms.dM[d];
                    }
                    pr.du_surf = du_surf;
                    G.audit_du = ff_value(accp) + ((sep ? ff_value(accr) : 0.0) + du_surf);
                    G.audit_pending = kind != FAU_MOVE_NONE && flags == 0 ? 1 : 0; // finite in both states
                    ms.prev_accept = 0; // the probe's pass folded the last accepted change
                }
            }
            break;
        }

        if (warp == 0) {
            accp = lane < NW ? red_a[lane] : FF{0.f, 0.f};
            accr = lane < NW ? red_b[lane] : FF{0.f, 0.f};
            scale = lane < NW ? red_s[lane] : 0.f;
            flags = lane < NW ? red_f[lane] : 0;
            if (maxe) {
                accn = lane < NW ? red_n[lane] : FF{0.f, 0.f};
                acco = lane < NW ? red_o[lane] : FF{0.f, 0.f};
            }
#pragma unroll
            for (int o = NW / 2; o > 0; o >>= 1) {
                FF ta{__shfl_xor_sync(0xffffffffu, accp.hi, o), __shfl_xor_sync(0xffffffffu, accp.lo, o)};
                accp = ff_sum(accp, ta);
                if (maxe) {
                    FF tn{__shfl_xor_sync(0xffffffffu, accn.hi, o), __shfl_xor_sync(0xffffffffu, accn.lo, o)};
                    accn = ff_sum(accn, tn);
                    FF to{__shfl_xor_sync(0xffffffffu, acco.hi, o), __shfl_xor_sync(0xffffffffu, acco.lo, o)};
                    acco = ff_sum(acco, to);
                }
                if (sep) {
                    FF tb{__shfl_xor_sync(0xffffffffu, accr.hi, o), __shfl_xor_sync(0xffffffffu, accr.lo, o)};
                    accr = ff_sum(accr, tb);
                    scale += __shfl_xor_sync(0xffffffffu, scale, o);
                }
                flags |= __shfl_xor_sync(0xffffffffu, flags, o);
            }
            int accept = 0, stop = 0;
            double du = 0.0;
            if (lane == 0) {
                if (kind != FAU_MOVE_NONE) {
                    const double du_nb = ff_value(accp); // without detail or maxe: pair + reciprocal together
                    const double du_rec = sep ? ff_value(accr) : 0.0;
                    double du_surf = 0.0, m2o = 0.0;
                    if (S.flags & SYS_SURFACE) {
                        double m2n = 0.0;
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            const double mn = __dadd_rn(M[d], ms.dM[d]);
                            m2o = __dadd_rn(m2o, __dmul_rn(M[d], M[d]));
                            m2n = __dadd_rn(m2n, __dmul_rn(mn, mn));
                        }
                        du_surf = S.surf_pref * (m2n - m2o);
                    }
                    const double fin = du_nb + (du_rec + du_surf);
                    du = energy_change(fin, flags & F_NEW_INF, flags & F_OLD_INF, flags & F_NEW_NAN, flags & F_OLD_NAN);
                    if (maxe && flags == 0) {
                        // Hamiltonian::energy (src/energy.cpp:1227-1241) per state: self, Nonbonded,
                        // Ewald, summed up to the first term >= maxenergy.  Self is the same in
                        // both states; Nonbonded is this move's partial energy (new - old = du_nb)
                        const double Mx = S.maxenergy;
                        double self = 0.0;
                        if (S.flags & SYS_SELF)
                            for (int a = 0; a < m; a++) self += S.itype_self[ms.rec_new[a].w >> 24];
                        if ((S.flags & SYS_SELF) && !(self < Mx)) {
                            du = 0.0; // both sums end at the self term
                        }
                        else {
                            const double nn = ff_value(accn), no = nn - du_nb;
                            const bool tn = !(nn < Mx), to = !(no < Mx);
                            if (tn || to) {
                                // the Ewald term of each state (reciprocal + surface), absolute
                                const double eo = (S.flags & SYS_EWALD) ? ff_value(acco) + S.surf_pref * m2o : 0.0;
                                const double en = eo + (du_rec + du_surf);
                                du = du_nb + ((tn ? 0.0 : en) - (to ? 0.0 : eo));
                            }
                        }
                    }
                    const double x = du * S.beta_scale;
                    if (A.pending) { // evaluate only: the caller's Metropolis decides
                        PlainMove& P = *A.pending;
                        P.kind = kind;
                        P.first = ms.first;
                        P.m = m;
                        P.group = kind == FAU_MOVE_MOLECULAR ? ms.index : -1;
                        P.count_move = 0;
                        for (int a = 0; a < m; a++)
                            for (int d = 0; d < 3; d++) P.xn[a][d] = ms.xn[a][d];
                        for (int d = 0; d < 3; d++) {
                            P.cm_new[d] = ms.cm_new[d];
                            P.dM[d] = ms.dM[d];
                        }
                        P.du = du;
                    }
                    else if (isnan(x)) {
                        stop = FAU_ERR_NAN;
                    }
                    else {
                        accept = metropolis(x, ms.u) ? 1 : 0;
                    }
                    if (detail) {
                        fau_trial_result r;
                        r.du = du;
                        r.du_nonbonded = du_nb;
                        r.du_ewald = du_rec + du_surf;
                        r.err_scale = (double)scale;
                        r.accepted = accept;
                        r.new_inf = (flags & F_NEW_INF) ? 1 : 0;
                        r.old_inf = (flags & F_OLD_INF) ? 1 : 0;
                        r.pad = 0;
                        A.detail[poff + mv] = r;
                    }
                    if (accept) {
                        n_acc++;
                        sum_du += du;
                        energy += du;
#pragma unroll
                        for (int d = 0; d < 3; d++) M[d] = __dadd_rn(M[d], ms.dM[d]);
                    }
                    if (!stop) n_mv++;
                }
                if (A.acc_out) A.acc_out[poff + mv] = (uint8_t)accept;
                if (A.du_out) A.du_out[poff + mv] = du;
            }
            accept = __shfl_sync(0xffffffffu, accept, 0);
            stop = __shfl_sync(0xffffffffu, stop, 0);
            tick(4);
            if (stop) {
                if (lane == 0) {
                    ms.stop = stop;
                    ms.prev_accept = 0;
                    ms.consumed = mv;
                }
            }
            else {
                // ---- commit (State::sync trial -> accepted): positions, records, cells, mass centre
                if (accept) {
                    if (lane < m) {
                        const int i = ms.first + lane;
                        S.x[i] = ms.xn[lane][0];
                        S.y[i] = ms.xn[lane][1];
                        S.z[i] = ms.xn[lane][2];
                        S.rec[i] = ms.rec_new[lane];
                    }
                    if (lane == 0) {
                        if (kind == FAU_MOVE_MOLECULAR) {
                            const int g = ms.index;
#pragma unroll
                            for (int d = 0; d < 3; d++) S.g_cm[3 * g + d] = ms.cm_new[d];
                            S.g_cmrec[g] = ms.cmrec_new;
                        }
                        else if (S.flags & SYS_CELLS) {
                            const int i = ms.index;
                            const int co = ms.cell_old, cn = ms.cell_new;
                            const int so = S.slot_of[i];
                            if (co == cn) {
                                S.cell_rec[(size_t)co * S.cap + so] = ms.rec_new[0];
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
                                    // keep the particle listed in its old cell: the host regrows the list
                                    S.cell_rec[(size_t)co * S.cap + last] = ms.rec_new[0];
                                    S.slot_of[i] = last;
                                    S.cell_cnt[co] = last + 1;
                                    stop = FAU_ERR_CAPACITY;
                                }
                                else {
                                    S.cell_rec[(size_t)cn * S.cap + sn] = ms.rec_new[0];
                                    S.cell_cnt[cn] = sn + 1;
                                    S.cell_of[i] = cn;
                                    S.slot_of[i] = sn;
                                }
                            }
                        }
                    }
                    stop = __shfl_sync(0xffffffffu, stop, 0);
                }
                __syncwarp();
                tick(5);
                if (stop) {
                    if (lane == 0) {
                        ms.stop = stop;
                        ms.prev_accept = accept;
                        ms.consumed = mv + 1;
                    }
                }
                else if (mv + 1 < nloop) {
                    // ---- prepare the next move (after the last: the audit probe)
                    const Proposal p = PHILOX ? philox_proposal(S, ctr0 + (unsigned long long)(mv + 1), sys_id, A.seed,
                                                                dp_f, dprot, molecular_sys)
                                              : load_proposal(A.props[poff + (mv + 1 < nmoves ? mv + 1 : nmoves - 1)]);
                    prepare_move(S, ms, p, lane, K ? tab : nullptr, nc);
                    if (lane == 0) {
                        if (mv + 1 == nmoves && ms.stop) { // no probe of an invalid proposal
                            ms.stop = 0;
                            ms.kind = FAU_MOVE_NONE;
                            ms.m = 0;
                        }
                        ms.prev_accept = accept;
                        ms.consumed = mv + 1;
                    }
                    __syncwarp();
                }
                else if (lane == 0) {
                    ms.prev_accept = accept;
                    ms.consumed = mv + 1;
                }
                tick(6);
            }
        }
        if (tid == 0 && A.time_budget_ns && global_ns() - sh_t0 >= A.time_budget_ns) sh_up_at = mv + 1;
        __syncthreads(); // B2
        tick(tid == 0 ? 7 : 10);
    }
    if (timing)
        for (int j = 0; j < kPhaseSlots; j++)
            if (tacc[j]) atomicAdd(&A.phase_cycles[blockIdx.x * kFastPhaseSlots + j], tacc[j]);

    // the pending changes stay pending: the next launch continues from them exactly as the next
    // move would (the host folds them into the master before it reads Q)
    for (int k = tid; k < K; k += NT) {
        S.qpend[k] = pend[k];
        S.qdlt[k] = dlt[k];
    }
    __shared__ unsigned long long red_u[NW][2];
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
        if (ms.stop) G.err = ms.stop;
        G.consumed = ms.stop ? ms.consumed : (sh_up_at >= 0 ? sh_up_at : nmoves);
        G.q_valid = K ? ms.prev_accept : 0;
        G.q_since = K ? since_flush : 0;
        G.cycles += (unsigned long long)(clock64() - t_start);
    }
}

// dynamic shared memory of a chain kernel for K k-vectors and table size nc
__host__ __device__ inline size_t chain_smem_bytes_v2(int K, int nc)
{
    return (size_t)K * (3 * sizeof(float2) + sizeof(int) + sizeof(float)) +
           (size_t)kTableAtoms * 6 * (2 * nc + 1) * sizeof(float2);
}

template <int NT, bool PH>
cudaError_t launch_chain_inst(const ChainArgs& a, int nblocks, int K, int nc, cudaStream_t st, bool prepare_only)
{
    // the dynamic allowance is raised on demand (the 48 KiB default also covers the static shared
    // memory), never inside a stream capture: callers prepare first
    static size_t granted = 0;
    const size_t smem = chain_smem_bytes_v2(K, nc);
    if (smem > granted || granted == 0) {
        cudaError_t e = cudaFuncSetAttribute(chain_kernel<NT, PH>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        granted = smem;
    }
    if (prepare_only) return cudaSuccess;
    chain_kernel<NT, PH><<<nblocks, NT, smem, st>>>(a);
    return cudaGetLastError();
}

} // namespace fau
