// fau_dev.cuh -- device-side layout and arithmetic helpers of the GB300
// Metropolis MC hot path.
//
// Layout in HBM, per system (one Faunus Space + Hamiltonian):
//   x, y, z       FP64 master positions (SoA).  All move arithmetic that
//                 decides where a particle ends up is FP64 and IEEE-exact
//                 (__dadd_rn / __dmul_rn: never contracted), so the chain
//                 is bit-identical to the FP64 oracle under the same RNG.
//   rec           uint4 {ux, uy, uz, (itype << 24) | index}: fixed-point
//                 copy with 2^32 units per box length.  Integer subtraction
//                 of two records is the minimum-image separation (exact),
//                 and n.u mod 2^32 is the exact reduced Ewald phase.
//   cell_rec      the same records bucketed by cell: `cap` slots per cell
//                 (a power of two), the first cell_cnt[c] in use, the rest
//                 holding .w = kEmptySlot; cell_of, slot_of: where each
//                 particle is listed.  Updated incrementally on every accept.
//   Q             Ewald structure factor, FP64 complex master copy.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/fau_gpu.h"

namespace fau {

constexpr int kMaxITypes = 16;     // internal (type, charge) classes per system
constexpr int kMaxGroupAtoms = 32; // atoms moved together in one molecular move
constexpr int kFlushAccepts = 64;  // FP32 pending Q deltas flushed to FP64 every N accepts
constexpr uint32_t kEmptySlot = 0xFFFFFFFFu; // .w of a cell-list slot at or beyond the cell's count

enum SysFlags : int {
    SYS_CELLS = 1 << 0,   // single-atom moves use the cell list
    SYS_EWALD = 1 << 1,
    SYS_SURFACE = 1 << 2, // Ewald surface term active (epss >= 1)
    SYS_SELF = 1 << 3,    // ParticleSelfEnergy present
    SYS_OCC = 1 << 4,     // the pipelined kernel stages the occupied slots of stencil cells only
    SYS_SPREAD = 1 << 5,  // ... with the stencil's cells spread over all compute warps (dense cells)
};

// pair parameters for one (itype a, itype b) class pair, FP32
struct PairF {
    float s2, e4, hs2, qq; // sigma^2, 4 eps, hard-sphere sigma^2, lB qa qb
};

// FAU_PAIR_SPLINE table of one (itype a, itype b) class pair (the atom types' KnotData)
struct SplineP {
    double zmin_d, zmax_d; // first and last knot (r^2), FP64
    float zmin, zmax;      // the same, FP32 (round to nearest)
    float inv_h;           // index-grid cells per unit r^2 over [zmin, zmax]
    int knot0;             // first knot in spl_zf / spl_zd
    int coef0;             // first coefficient in spl_cf / spl_cd (6 a piece)
    int pieces;            // knots - 1
    int grid0, grid_n;     // index grid in spl_grid: the piece holding each cell's start
    int hs;                // +inf at r^2 <= zmin (hardsphere_repulsion)
    int pad;
};
constexpr int kSplineGrid = 256; // index-grid cells a pair (at most)

struct DevSys {
    // geometry (cuboid)
    double L[3], half[3], inv[3];
    double fx_scale[3]; // 2^32 / L : FP64 -> fixed point
    float fx_len[3];    // L / 2^32 : fixed point -> FP32 angstrom
    double fx_lend[3];  // L / 2^32 in FP64
    float inv_f[3];     // 1 / L in FP32
    int knc;            // largest |n| component of the k-vectors (phase table half-width)
    int n, n_groups, flags, pad0;

    double* x;
    double* y;
    double* z;
    uint4* rec;
    int* group_of;
    float* itype_q;     // charge per internal type (FP32)
    double* itype_qd;   // FP64
    double* itype_self; // self energy per internal type (kT)
    int itype_type[kMaxITypes]; // atom type id (Particle::id) of each internal type

    // groups
    int* g_begin;     // n_groups + 1
    int* g_flags;
    double* g_cm;     // n_groups * 3 FP64 mass centres
    uint4* g_cmrec;   // fixed-point mass centres
    int* atomic_idx;  // particles of atomic groups (for molecular moves)
    int n_atomic;

    // pair potential
    int nt, terms, coul_type, pad1;
    float lB, rc_coul, rc2_coul, alpha;
    float rc2_pair;   // 0: no truncation
    double rc2_pair_d, rc_coul_d, alpha_d, lB_d;
    // FAU_COUL_TRUNC: S(q) = cerfc erfc(alpha r) + sum_k cpoly[k] q^k, q = r / Rc
    int npoly;
    float cerfc, inv_rc;
    float cpoly[FAU_COUL_MAX_POLY];
    double cerfc_d, inv_rc_d;
    double cpoly_d[FAU_COUL_MAX_POLY];
    double cut_g2g2;  // group mass-centre cutoff^2 (FP64); < 0: none (with n_mol > 0: >= 0 if any pair has one)
    float cut_g2g2f;
    int n_mol;        // > 0: per molecule-kind pair cutoffs^2 below, indexed by g_molid
    int* g_molid;     // n_groups molecule kinds (n_mol > 0 only)
    double* cut2_mol; // n_mol^2 cutoffs^2 (FP64); < 0: no cutoff for that pair
    float* cut2_molf; // FP32 copies
    // mass-centre cells of the molecular groups (the molecular kernel's GroupCutoff candidates),
    // at least as wide as the largest group cutoff; rebuilt at each launch of that kernel
    int gdim[3], gncell;  // gncell 0: every group is a candidate
    int gcap, gshift;     // slots a cell (a power of two >= 32) and its log2
    double ginv[3];       // cells per unit length
    int* gc_cnt;          // gncell counts
    int* gc_list;         // gncell * gcap group indices, ascending within a cell
    PairF* pair;      // nt*nt
    double* pair_d;   // nt*nt*4 FP64 copies (s2, e4, hs2, qq)
    // FAU_PAIR_SPLINE: tables per class pair (nt*nt SplineP), knots and coefficients
    SplineP* spl;
    float* spl_zf;
    double* spl_zd;
    float* spl_cf;
    double* spl_cd;
    int* spl_grid;

    // cell list
    int cdim[3], ncell;
    int off_min[3], off_max[3];
    int cap, pad2;
    // reciprocal multipliers of cdim[0] and cdim[0] cdim[1] (cell index -> coordinates by
    // multiply-high, exact while ncell times the divisor stays below 2^32); 0: divide.  Set by the
    // pipelined kernel in its shared copy of the descriptor
    uint32_t cmag0, cmag01;
    double cell_len[3];
    int* cell_cnt;
    uint4* cell_rec;
    int* cell_of;
    int* slot_of;

    // Ewald
    int K, pad3;
    int* kn;          // packed (nx+128) | (ny+128)<<8 | (nz+128)<<16
    float* Ak;
    double* Akd;
    double2* Q;       // FP64 master
    // accepted Q(k) changes not yet flushed into the master, kept across launches so that a chain
    // split into several launches evolves exactly as in one (Q = master + qpend [+ qdlt if q_valid])
    float2* qpend;    // FP32 pending sums
    float2* qdlt;     // the last accepted move's change, folded into qpend by the next move
    int q_valid, q_since; // qdlt pending; accepts since the last flush into the master
    double rec_pref;  // 2 pi lB / V
    double surf_pref; // const_inf 2 pi lB / ((2 epss + 1) V)
    double M[3];      // sum q r (surface term)

    // running state
    double energy;     // running total energy (kT), FP64 (see sys_energy)
    double beta_scale; // multiplies dU in the Metropolis test (PT temperature ladder)
    int err;           // fau_status raised on the device
    int pad4;
    float e_acc_hi, e_acc_lo; // the pipelined kernel's float-float sum of accepted changes not yet in `energy`
    unsigned long long moves, accepted, pair_evals, k_updates;
    double sum_du;
    long long consumed; // proposals performed by the last chain launch
    unsigned long long cycles; // SM clock cycles spent in chain launches (summed)
    // the pipelined kernel's audit: the largest error of its FP32 energy changes against FP64
    // re-evaluations of its probe moves, relative to max(|dU|, S) and to |dU| (|dU| > 1e-3 kT),
    // and the probes evaluated, since the system was made
    double audit_scaled_max, audit_rel_max;
    unsigned long long audit_samples;
    // the last probe's record (kAuditRecBytes, device; NULL: no audit) and its FP32 energy change
    unsigned char* audit_rec;
    double audit_du;
    int audit_pending, pad5;
    // Hamiltonian maxenergy (src/energy.cpp:1227-1241): maxe 1 when finite; the chain kernel then
    // sums each state's terms (self, Nonbonded, Ewald) up to the first >= maxenergy
    double maxenergy;
    int maxe, pad6;
};
constexpr size_t kAuditRecBytes = 1024; // a probe move: the pipelined kernel's FastMove or a ProbeRecord

// the probe move of the molecular kernel or the chain kernel: its kind, the group (molecular) or
// particle (single atom) it moves, the moved atoms' trial positions (the old ones are the
// system's, unchanged by the probe), the new mass centre and the dipole change
struct ProbeRecord {
    int kind, index, m, first;
    double cm_new[3], dM[3], du_surf, pad;
    double xn[kMaxGroupAtoms][3];
};
static_assert(sizeof(ProbeRecord) <= kAuditRecBytes, "audit record size");

// ---------------------------------------------------------------- fixed point
__host__ __device__ inline uint32_t to_fixed(double x, double scale)
{
#ifdef __CUDA_ARCH__
    const double t = __dmul_rn(x, scale);
    return (uint32_t)(unsigned long long)__double2ll_rn(t);
#else
    const double t = x * scale;
    return (uint32_t)(unsigned long long)llrint(t);
#endif
}

// ---------------------------------------------------------------- compensated sums
// float-float accumulator (Knuth TwoSum): ~48-bit significand, FP32 pipe only.
struct FF {
    float hi, lo;
};
__device__ __forceinline__ void ff_add(FF& a, float b)
{
    const float s = __fadd_rn(a.hi, b);
    const float bb = __fsub_rn(s, a.hi);
    const float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    a.hi = s;
    a.lo = __fadd_rn(a.lo, e);
}
__device__ __forceinline__ FF ff_sum(FF a, FF b)
{
    const float s = __fadd_rn(a.hi, b.hi);
    const float bb = __fsub_rn(s, a.hi);
    float e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
    e = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
    const float hi = __fadd_rn(s, e);
    const float lo = __fsub_rn(e, __fsub_rn(hi, s));
    return {hi, lo};
}
__device__ __forceinline__ double ff_value(FF a) { return (double)a.hi + (double)a.lo; }

// ---------------------------------------------------------------- Philox4x32-10
// Counter-based RNG of Salmon, Moraes, Dror & Shaw (SC'11), published constants.
struct U4 {
    uint32_t x, y, z, w;
};
__device__ __forceinline__ U4 philox(U4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        const uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = {hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}
__device__ __forceinline__ double u01_53(uint32_t a, uint32_t b) // [0,1) with 53 bits
{
    const unsigned long long v = ((unsigned long long)(a >> 5) << 26) | (b >> 6);
    return (double)v * (1.0 / 9007199254740992.0);
}
__device__ __forceinline__ float u01_24(uint32_t a) { return (float)(a >> 8) * (1.0f / 16777216.0f); }

// ---------------------------------------------------------------- exact conversions on the integer pipe
// GB300's FP64 pipe issues about one warp instruction per 64 cycles, so the per-move
// path builds doubles from their bit patterns where the value is exact anyway.

// float -> double, exact (normal, subnormal, zero, inf, NaN)
__device__ __forceinline__ double f2d_bits(float f)
{
    const uint32_t b = __float_as_uint(f);
    const uint32_t e = (b >> 23) & 0xFFu, m = b & 0x7FFFFFu;
    unsigned long long r = (unsigned long long)(b >> 31) << 63;
    if (e == 0xFFu) {
        r |= 0x7FF0000000000000ULL | ((unsigned long long)m << 29);
    }
    else if (e != 0u) {
        r |= ((unsigned long long)(e + 896u) << 52) | ((unsigned long long)m << 29);
    }
    else if (m != 0u) { // subnormal: m 2^-149 with the leading bit at position p
        const int p = 31 - __clz((int)m);
        r |= ((unsigned long long)(p - 149 + 1023) << 52) | (((unsigned long long)m << (52 - p)) & 0xFFFFFFFFFFFFFULL);
    }
    return __longlong_as_double((long long)r);
}

// v 2^-53 for an integer 0 <= v < 2^53, exact
__device__ __forceinline__ double u53_bits(unsigned long long v)
{
    if (v == 0ull) return 0.0;
    const int p = 63 - __clzll((long long)v);
    const unsigned long long r = ((unsigned long long)(p - 53 + 1023) << 52) | ((v << (52 - p)) & 0xFFFFFFFFFFFFFULL);
    return __longlong_as_double((long long)r);
}

// a finite double truncated to float (relative error below 2^-23; magnitudes below
// 2^-126 give a signed zero, above the float range an infinity)
__device__ __forceinline__ float d2f_trunc(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const uint32_t sign = (uint32_t)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if (e <= 0) return __uint_as_float(sign);
    if (e >= 255) return __uint_as_float(sign | 0x7F800000u);
    return __uint_as_float(sign | ((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu));
}

// a double in [0, 1] truncated to float (relative error below 2^-23; values below 2^-126 give 0)
__device__ __forceinline__ float d2f_trunc01(double u)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(u);
    const int e = (int)((b >> 52) & 0x7FF) - 1023 + 127;
    if ((long long)b <= 0 || e <= 0) return 0.f;
    if (e >= 255) return __uint_as_float(0x7F800000u);
    return __uint_as_float(((uint32_t)e << 23) | (uint32_t)((b >> 29) & 0x7FFFFFu));
}

// ---------------------------------------------------------------- geometry, FP64 exact
// Chameleon::boundary (reference src/geometry.h:407-427) with anint (:132-135).
__device__ __forceinline__ double boundary1(double a, double L, double half, double inv)
{
    // |a| > half (half > 0) compared as bit patterns on the integer pipe: an FP64 compare is an
    // FP64-pipe instruction, one warp instruction per 64 cycles on this GPU (NaN takes the branch
    // and stays NaN, as it does untouched)
    if ((__double_as_longlong(a) & 0x7FFFFFFFFFFFFFFFLL) > __double_as_longlong(half)) {
        const double t = __dmul_rn(a, inv);
        const int n = (int)(t > 0.0 ? __dadd_rn(t, 0.5) : __dsub_rn(t, 0.5));
        a = __dsub_rn(a, __dmul_rn(L, (double)n));
    }
    return a;
}
// Chameleon::sqdist (src/geometry.h:460-485), summed ((x^2 + y^2) + z^2)
__device__ __forceinline__ double sqdist_d(const DevSys& S, const double* a, const double* b)
{
    double d[3];
#pragma unroll
    for (int k = 0; k < 3; k++) {
        const double v = fabs(__dsub_rn(a[k], b[k]));
        d[k] = __dsub_rn(v, v > S.half[k] ? S.L[k] : 0.0);
    }
    return __dadd_rn(__dadd_rn(__dmul_rn(d[0], d[0]), __dmul_rn(d[1], d[1])), __dmul_rn(d[2], d[2]));
}

// GroupCutoff::getCutoff(molid1, molid2)^2 of two groups (src/energy.h:740-768); < 0: none
__device__ __forceinline__ double group_cut2(const DevSys& S, int g1, int g2)
{
    return S.n_mol > 0 ? S.cut2_mol[S.g_molid[g1] * S.n_mol + S.g_molid[g2]] : S.cut_g2g2;
}

// the running total energy: the FP64 sum plus the pipelined kernel's unfolded float-float part,
// which stays unfolded across launches (a chain split into launches sums as in one)
__host__ __device__ inline double sys_energy(const DevSys& S)
{
    return S.energy + ((double)S.e_acc_hi + (double)S.e_acc_lo);
}

// squared minimum-image distance of two fixed-point records, FP32
// the GPU's global nanosecond timer (PTX %globaltimer)
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ float r2_fixed(const DevSys& S, uint4 a, uint4 b)
{
    const float dx = (float)(int32_t)(a.x - b.x) * S.fx_len[0];
    const float dy = (float)(int32_t)(a.y - b.y) * S.fx_len[1];
    const float dz = (float)(int32_t)(a.z - b.z) * S.fx_len[2];
    return fmaf(dx, dx, fmaf(dy, dy, dz * dz));
}

// ---------------------------------------------------------------- pair energy, FP32
// The enabled terms at FP32 r^2 with the cutoff decisions already made (in_pair: inside
// the pair cutoff; in_coul: inside the Coulomb cutoff; overlap: hard-sphere contact).
__device__ __forceinline__ float pair_core(const DevSys& S, const PairF& p, float r2, bool in_pair, bool in_coul,
                                           bool overlap, bool& inf, bool& nan, float& mag)
{
    const int terms = S.terms;
    if (!in_pair) return 0.f;
    float u = 0.f, m = 0.f;
    if (terms & FAU_PAIR_COULOMB) {
        float c = 0.f;
        if (S.coul_type == FAU_COUL_PLAIN) {
            c = p.qq * rsqrtf(r2);
        }
        else if (in_coul) {
            if (S.coul_type == FAU_COUL_EWALD) {
                // erfc amplifies argument errors by ~2 (alpha r)^2: correctly rounded r and 1/r
                const float r = __fsqrt_rn(r2);
                c = p.qq * erfcf(S.alpha * r) * __frcp_rn(r);
            }
            else if (S.coul_type == FAU_COUL_TRUNC) {
                // Horner in q; the error scale is |qq/r| (|e| erfc + sum |c_k| q^k)
                const float r = __fsqrt_rn(r2), q = r * S.inv_rc, ir = __frcp_rn(r);
                float sp = 0.f, sa = 0.f;
                for (int k = S.npoly - 1; k >= 0; k--) {
                    sp = fmaf(sp, q, S.cpoly[k]);
                    sa = fmaf(sa, q, fabsf(S.cpoly[k]));
                }
                float e = 0.f;
                if (S.cerfc != 0.f) e = S.cerfc * erfcf(S.alpha * r);
                const float pq = p.qq * ir;
                u += pq * (sp + e);
                m += fabsf(pq) * (sa + fabsf(e));
            }
            else {
                c = p.qq * rsqrtf(r2);
            }
        }
        u += c;
        m += fabsf(c);
    }
    if (terms & (FAU_PAIR_LJ | FAU_PAIR_WCA)) {
        // (s/r)^6 from the correctly rounded 1/r^2: x^6 - x^3 cancels near the LJ
        // minimum, so the approximate rsqrt would cost ~10x the error
        float x = p.s2 * __frcp_rn(r2);
        x = x * x * x;
        // error scale: the r^-12 and r^-6 parts separately (they cancel near r = sigma)
        if (terms & FAU_PAIR_LJ) {
            u += p.e4 * (x * x - x);
            m += fabsf(p.e4) * (x * x + x);
        }
        if ((terms & FAU_PAIR_WCA) && !(r2 > p.s2 * 1.2599210498948732f)) {
            u += p.e4 * (x * x - x + 0.25f);
            m += fabsf(p.e4) * (x * x + x + 0.25f);
        }
    }
    if (overlap) inf = true;
    if (!isfinite(u)) {
        if (isnan(u) && !(p.s2 == p.s2)) nan = true; // missing coefficients (NaN sigma)
        else inf = true;                              // FP32 overflow at r -> 0
        u = 0.f;
        m = 0.f;
    }
    mag += m;
    return u;
}

// N pairs away from every guard band at once, each with exactly pair_u32_far's arithmetic;
// the loop over the pairs sits inside each term (and every per-pair condition is a
// select), so the N dependency chains interleave instead of running one after another.
// lj[j] false: the LJ/WCA terms of pair j are skipped -- only where they are exactly zero
// (4 eps = 0, sigma finite, r^2 far enough from 0 that (s/r)^12 cannot overflow).
template <int N>
__device__ __forceinline__ void pair_far_multi(const DevSys& S, const PairF* p, const float* r2, float* u, bool* inf,
                                               bool* nan, const bool* lj)
{
    const int terms = S.terms;
    float uu[N], mm[N];
#pragma unroll
    for (int j = 0; j < N; j++) {
        uu[j] = 0.f;
        mm[j] = 0.f;
    }
    if (terms & FAU_PAIR_COULOMB) {
        if (S.coul_type == FAU_COUL_PLAIN) {
#pragma unroll
            for (int j = 0; j < N; j++) {
                const float c = p[j].qq * rsqrtf(r2[j]);
                uu[j] += c;
                mm[j] += fabsf(c);
            }
        }
        else if (S.coul_type == FAU_COUL_EWALD) {
#pragma unroll
            for (int j = 0; j < N; j++) {
                const float r = __fsqrt_rn(r2[j]);
                const float cv = p[j].qq * erfcf(S.alpha * r) * __frcp_rn(r);
                const float c = r2[j] < S.rc2_coul ? cv : 0.f;
                uu[j] += c;
                mm[j] += fabsf(c);
            }
        }
        else if (S.coul_type == FAU_COUL_TRUNC) {
#pragma unroll
            for (int j = 0; j < N; j++) {
                const float r = __fsqrt_rn(r2[j]), q = r * S.inv_rc, ir = __frcp_rn(r);
                float sp = 0.f, sa = 0.f;
                for (int k = S.npoly - 1; k >= 0; k--) {
                    sp = fmaf(sp, q, S.cpoly[k]);
                    sa = fmaf(sa, q, fabsf(S.cpoly[k]));
                }
                float e = 0.f;
                if (S.cerfc != 0.f) e = S.cerfc * erfcf(S.alpha * r);
                const float pq = p[j].qq * ir;
                const bool in = r2[j] < S.rc2_coul;
                uu[j] += in ? pq * (sp + e) : 0.f;
                mm[j] += in ? fabsf(pq) * (sa + fabsf(e)) : 0.f;
                uu[j] += 0.f; // the c = 0 term of the other forms
            }
        }
        else {
#pragma unroll
            for (int j = 0; j < N; j++) {
                const float c = r2[j] < S.rc2_coul ? p[j].qq * rsqrtf(r2[j]) : 0.f;
                uu[j] += c;
                mm[j] += fabsf(c);
            }
        }
    }
    if (terms & (FAU_PAIR_LJ | FAU_PAIR_WCA)) {
#pragma unroll
        for (int j = 0; j < N; j++) {
            if (!lj[j]) continue;
            float x = p[j].s2 * __frcp_rn(r2[j]);
            x = x * x * x;
            if (terms & FAU_PAIR_LJ) {
                uu[j] += p[j].e4 * (x * x - x);
                mm[j] += fabsf(p[j].e4) * (x * x + x);
            }
            if (terms & FAU_PAIR_WCA) {
                const bool in = !(r2[j] > p[j].s2 * 1.2599210498948732f);
                uu[j] += in ? p[j].e4 * (x * x - x + 0.25f) : 0.f;
                mm[j] += in ? fabsf(p[j].e4) * (x * x + x + 0.25f) : 0.f;
            }
        }
    }
#pragma unroll
    for (int j = 0; j < N; j++) {
        const bool in_pair = !(S.rc2_pair > 0.f && r2[j] >= S.rc2_pair);
        const bool overlap = (terms & FAU_PAIR_HS) && r2[j] < p[j].hs2;
        bool fi = in_pair && overlap, fn = false;
        float v = in_pair ? uu[j] : 0.f;
        if (in_pair && !isfinite(v)) {
            if (isnan(v) && !(p[j].s2 == p[j].s2)) fn = true;
            else fi = true;
            v = 0.f;
        }
        u[j] = v;
        inf[j] = fi;
        nan[j] = fn;
    }
}

// Whether FP32 r^2 lies within the 1e-5 guard band of a cutoff or contact distance, where
// the FP64 distance decides (pair_u32).
__device__ __forceinline__ bool pair_near(const DevSys& S, const PairF& p, float r2)
{
    const int terms = S.terms;
    const bool cut_coul = (terms & FAU_PAIR_COULOMB) && S.coul_type != FAU_COUL_PLAIN;
    return (S.rc2_pair > 0.f && fabsf(r2 - S.rc2_pair) <= 1e-5f * S.rc2_pair) ||
           (cut_coul && fabsf(r2 - S.rc2_coul) <= 1e-5f * S.rc2_coul) ||
           ((terms & FAU_PAIR_HS) && fabsf(r2 - p.hs2) <= 1e-5f * p.hs2);
}

// A pair away from every guard band (pair_near false): the FP32 decisions are exact.
__device__ __forceinline__ float pair_u32_far(const DevSys& S, const PairF& p, float r2, bool& inf, bool& nan,
                                              float& mag)
{
    const bool in_pair = !(S.rc2_pair > 0.f && r2 >= S.rc2_pair);
    const bool in_coul = r2 < S.rc2_coul;
    const bool overlap = (S.terms & FAU_PAIR_HS) && r2 < p.hs2;
    return pair_core(S, p, r2, in_pair, in_coul, overlap, inf, nan, mag);
}

// FAU_PAIR_SPLINE, FP32: the piece z_i < r2 <= z_{i+1} (Andrea::eval's lower_bound,
// src/tabulate.h:188-207) from the index grid and a short scan either way, then Horner in
// dz = r2 - z_i. `mag` gets sum_k |c_k| |dz|^k, the error scale of the evaluation.
// Not inlined: the kernels keep the register allocation of the unsplined terms.
static __device__ __noinline__ float spline_u32(const DevSys& S, const SplineP& q, float r2, float& mag)
{
    int g = (int)((r2 - q.zmin) * q.inv_h);
    g = min(max(g, 0), q.grid_n - 1);
    int i = S.spl_grid[q.grid0 + g];
    const float* z = S.spl_zf + q.knot0;
    while (i > 0 && !(r2 > z[i])) i--;
    while (i < q.pieces - 1 && r2 > z[i + 1]) i++;
    const float* c = S.spl_cf + q.coef0 + 6 * i;
    const float dz = r2 - z[i], adz = fabsf(dz);
    float s = 0.f, a = 0.f;
#pragma unroll
    for (int k = 5; k > 0; k--) {
        s = dz * (s + c[k]);
        a = adz * (a + fabsf(c[k]));
    }
    mag += a + fabsf(c[0]);
    return s + c[0];
}

// FAU_PAIR_SPLINE, FP64 (totals and the plain form): lower_bound over the FP64 knots; absolute:
// the magnitude sum_k |c_k| |dz|^k instead (the error scale of the evaluation)
__device__ __forceinline__ double spline_u64(const DevSys& S, const SplineP& q, double r2, bool absolute = false)
{
    const double* z = S.spl_zd + q.knot0;
    int first = 0, count = q.pieces + 1;
    while (count > 0) {
        const int step = count / 2;
        if (z[first + step] < r2) {
            first += step + 1;
            count -= step + 1;
        }
        else {
            count = step;
        }
    }
    const int i = min(max(first - 1, 0), q.pieces - 1);
    const double* c = S.spl_cd + q.coef0 + 6 * i;
    const double dz = absolute ? fabs(r2 - z[i]) : r2 - z[i];
    double s = 0.0;
    for (int k = 5; k > 0; k--) s = dz * (s + (absolute ? fabs(c[k]) : c[k]));
    return s + (absolute ? fabs(c[0]) : c[0]);
}

// Sum of enabled terms (coulomb, LJ, WCA, HS).  Hard-sphere overlap and FP32
// overflow set `inf` instead of adding +inf, so the compensated sums stay finite.
// The terms are discontinuous at the pair cutoff, the Coulomb cutoff and the
// hard-sphere contact; when the FP32 distance is within 1e-5 (relative) of one of
// them, the reference FP64 distance (sqdist of the FP64 positions xi and particle
// j) decides which side the pair is on, so inclusion matches the FP64 oracle.
// `xj` (optional) replaces particle j's resident FP64 position when the caller
// knows a newer one than memory holds.  `mag` accumulates the sum of |summand|
// over the enabled terms, LJ's r^-12 and r^-6 parts counted separately (the
// floating-point error scale of this pair energy).  SPL false leaves out the
// FAU_PAIR_SPLINE tables (for callers that dispatch splined systems elsewhere).
template <bool SPL = true>
__device__ __forceinline__ float pair_u32(const DevSys& S, const PairF& p, int pidx, float r2, const double* xi,
                                          int j, bool& inf, bool& nan, float& mag, const double* xj = nullptr)
{
    const int terms = S.terms;
    bool in_pair = !(S.rc2_pair > 0.f && r2 >= S.rc2_pair);
    bool in_coul = r2 < S.rc2_coul;
    bool overlap = (terms & FAU_PAIR_HS) && r2 < p.hs2;
    auto r2_fp64 = [&]() {
        const double xr[3] = {xj ? xj[0] : S.x[j], xj ? xj[1] : S.y[j], xj ? xj[2] : S.z[j]};
        return sqdist_d(S, xi, xr);
    };
    if (pair_near(S, p, r2)) {
        const double r2d = r2_fp64();
        in_pair = !(S.rc2_pair_d > 0.0 && r2d >= S.rc2_pair_d);
        in_coul = __dadd_rn(sqrt(r2d), 2.220446049250313e-16) < S.rc_coul_d;
        overlap = (terms & FAU_PAIR_HS) && r2d < S.pair_d[4 * pidx + 2];
    }
    if (SPL && (terms & FAU_PAIR_SPLINE)) { // SplinedPotential::operator() src/potentials.h:807-823
        if (!in_pair) return 0.f;
        const SplineP& q = S.spl[pidx];
        bool above = r2 >= q.zmax, inside = r2 > q.zmin;
        if (fabsf(r2 - q.zmax) <= 1e-5f * q.zmax || fabsf(r2 - q.zmin) <= 1e-5f * q.zmin) {
            const double r2d = r2_fp64(); // the table's ends decide on the FP64 distance
            above = r2d >= q.zmax_d;
            inside = r2d > q.zmin_d;
        }
        if (above) return 0.f;
        if (inside) return spline_u32(S, q, r2, mag);
        if (q.hs) {
            inf = true;
            return 0.f;
        }
        // at or below the first knot: the exact terms
    }
    return pair_core(S, p, r2, in_pair, in_coul, overlap, inf, nan, mag);
}

// FAU_COUL_TRUNC short-range function in FP64: e erfc(alpha r) + Horner in q = r / Rc
__device__ __forceinline__ double coul_trunc_s(const DevSys& S, double r, bool absolute = false)
{
    const double q = r / S.rc_coul_d;
    double s = 0.0;
    for (int k = S.npoly - 1; k >= 0; k--) s = s * q + (absolute ? fabs(S.cpoly_d[k]) : S.cpoly_d[k]);
    if (S.cerfc_d != 0.0) s += (absolute ? fabs(S.cerfc_d) : S.cerfc_d) * erfc(S.alpha_d * r);
    return s;
}

// FP64 pair energy (plain form and total energy), same term order as the oracle
__device__ __forceinline__ double pair_u64(const DevSys& S, int ta, int tb, double r2)
{
    if (S.rc2_pair_d > 0.0 && r2 >= S.rc2_pair_d) return 0.0;
    if (S.terms & FAU_PAIR_SPLINE) {
        const SplineP& q = S.spl[ta * S.nt + tb];
        if (r2 >= q.zmax_d) return 0.0;
        if (r2 > q.zmin_d) return spline_u64(S, q, r2);
        if (q.hs) return __longlong_as_double(0x7ff0000000000000ULL);
    }
    const double* P = S.pair_d + 4 * (ta * S.nt + tb);
    const double s2 = P[0], e4 = P[1], hs2 = P[2], qq = P[3];
    double u = 0.0;
    if (S.terms & FAU_PAIR_COULOMB) {
        if (S.coul_type == FAU_COUL_PLAIN) {
            u += qq / sqrt(r2);
        }
        else {
            const double r = sqrt(r2) + 2.220446049250313e-16;
            if (r < S.rc_coul_d) {
                double s = 1.0;
                if (S.coul_type == FAU_COUL_EWALD) s = erfc(S.alpha_d * r);
                else if (S.coul_type == FAU_COUL_TRUNC) s = coul_trunc_s(S, r);
                u += qq / r * s;
            }
        }
    }
    if (S.terms & FAU_PAIR_LJ) {
        double x = s2 / r2;
        x = x * x * x;
        u += e4 * (x * x - x);
    }
    if (S.terms & FAU_PAIR_WCA) {
        double w = 0.0;
        if (!(r2 > s2 * 1.2599210498948732)) {
            double x = s2 / r2;
            x = x * x * x;
            w = e4 * (x * x - x + 0.25);
        }
        u += w;
    }
    if ((S.terms & FAU_PAIR_HS) && r2 < hs2) u += __longlong_as_double(0x7ff0000000000000ULL);
    return u;
}

// The error scale of a pair energy in FP64, as the parity tolerance defines it: the sum of
// |summand| over the enabled terms, the r^-12 and r^-6 parts of LJ / WCA counted separately (they
// cancel near r = sigma, where the rounding of any evaluation scales with their sum); the
// truncated-Coulomb polynomial by its |coefficients|; a splined pair by sum_k |c_k| |dz|^k.
__device__ __forceinline__ double pair_mag64(const DevSys& S, int ta, int tb, double r2)
{
    if (S.rc2_pair_d > 0.0 && r2 >= S.rc2_pair_d) return 0.0;
    const int ab = ta * S.nt + tb;
    if (S.terms & FAU_PAIR_SPLINE) {
        const SplineP& q = S.spl[ab];
        if (r2 >= q.zmax_d) return 0.0;
        if (r2 > q.zmin_d) return spline_u64(S, q, r2, true);
        if (q.hs) return 0.0;
    }
    const double* P = S.pair_d + 4 * ab;
    const double s2 = P[0], e4 = fabs(P[1]), qq = P[3];
    double m = 0.0;
    if (S.terms & FAU_PAIR_COULOMB) {
        if (S.coul_type == FAU_COUL_PLAIN) {
            m += fabs(qq / sqrt(r2));
        }
        else {
            const double r = sqrt(r2) + 2.220446049250313e-16;
            if (r < S.rc_coul_d) {
                double sv = 1.0;
                if (S.coul_type == FAU_COUL_EWALD) sv = erfc(S.alpha_d * r);
                else if (S.coul_type == FAU_COUL_TRUNC) sv = coul_trunc_s(S, r, true);
                m += fabs(qq / r * sv);
            }
        }
    }
    double x = s2 / r2;
    x = x * x * x;
    if (S.terms & FAU_PAIR_LJ) m += e4 * (x * x + x);
    if ((S.terms & FAU_PAIR_WCA) && !(r2 > s2 * 1.2599210498948732)) m += e4 * (x * x + x + 0.25);
    return isfinite(m) ? m : 0.0;
}

__device__ __forceinline__ void kn_unpack(int v, int& nx, int& ny, int& nz)
{
    nx = (v & 0xff) - 128;
    ny = ((v >> 8) & 0xff) - 128;
    nz = ((v >> 16) & 0xff) - 128;
}

// e^{i k.r} from a fixed-point record: the phase n.u mod 2^32 is exact.
__device__ __forceinline__ float2 eikr32(int nx, int ny, int nz, uint4 r)
{
    const uint32_t ph = (uint32_t)nx * r.x + (uint32_t)ny * r.y + (uint32_t)nz * r.z;
    const float t = (float)(int32_t)ph * 4.656612873077393e-10f; // 2^-31
    float s, c;
    sincospif(t, &s, &c);
    return make_float2(c, s);
}

} // namespace fau
