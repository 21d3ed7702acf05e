// fau_kernels.cu -- sm_103a kernels of the Metropolis MC energy hot path.
//
//   chain_kernel      persistent move loop, one CTA per Markov chain: proposal
//                     -> FP64 trial positions -> FP32 pair + Ewald dU with
//                     float-float sums -> FP64 Metropolis -> commit.  Replaces
//                     MetropolisMonteCarlo::performMove (src/montecarlo.cpp:139-187)
//                     for transrot / moltransrot moves.
//   total_pair_kernel FP64 Nonbonded pairing.all (src/energy.h:1290-1299).
//   q_rebuild_kernel  FP64 Q(k) = sum_j q_j e^{ik.r_j} (src/energy.cpp:191-206).
//   plain_*           the plain FP64 single-move form: one move per call,
//                     host-fed proposal and uniform (in-GPU comparison point).
#include "fau_dev.cuh"
#include "fau_kernels.h"

#include <cfloat>

namespace fau {

// ---------------------------------------------------------------- shared move state
struct MoveShared {
    int kind, index, m, first;
    int accept, stop, cell_old, cell_new;
    double u, du;
    double du_nb, du_ew, scale;
    int new_inf, old_inf, pad0, pad1;
    float q[kMaxGroupAtoms];
    float3 g[kMaxGroupAtoms]; // minimum-image displacement / L per moved atom (FP32, from FP64)
    uint4 rec_old[kMaxGroupAtoms];
    uint4 rec_new[kMaxGroupAtoms];
    double xn[kMaxGroupAtoms][3];
    double xo[kMaxGroupAtoms][3];
    double cm_new[3];
    double dM[3];
    uint4 cmrec_old, cmrec_new;
};

// cell of a position: fixed-point fast path, FP64 reference formula
// floor((x + L/2) / cell_len) (src/celllistimpl.h:139-143, src/sasa.cpp:466-468)
// whenever the position is within 2^-18 cell of a boundary -> bit-exact.
__device__ int cell_of_pos(const DevSys& S, const double* x, uint4 r)
{
    int c[3];
    const uint32_t u[3] = {r.x, r.y, r.z};
#pragma unroll
    for (int d = 0; d < 3; d++) {
        // shifted fixed point: [-L/2, L/2) -> [0, 2^32)
        const uint32_t s = u[d] + 0x80000000u;
        const unsigned long long prod = (unsigned long long)s * (unsigned long long)S.cdim[d];
        int v = (int)(prod >> 32);
        const uint32_t frac = (uint32_t)prod;
        if (frac < (1u << 14) || frac > 0xFFFFFFFFu - (1u << 14)) {
            const double t = __dadd_rn(x[d], __dmul_rn(0.5, S.L[d]));
            v = (int)floor(__ddiv_rn(t, S.cell_len[d]));
        }
        if (v < 0) v += S.cdim[d] * (abs(v) / S.cdim[d] + 1);
        else if (v >= S.cdim[d]) v -= S.cdim[d] * (v / S.cdim[d]);
        c[d] = v;
    }
    return c[0] + S.cdim[0] * (c[1] + S.cdim[1] * c[2]);
}

// GroupCutoff::cut (src/energy.h:761-768): sqdist(cm1, cm2) >= cutoff^2,
// FP32 on fixed-point mass centres, FP64 inside a 1e-5 guard band.
__device__ __forceinline__ bool group_cut(const DevSys& S, uint4 cmrec, const double* cm, int h)
{
    if (S.cut_g2g2 < 0.0) return false;
    const float r2 = r2_fixed(S, cmrec, S.g_cmrec[h]);
    if (r2 < S.cut_g2g2f * 0.99999f) return false;
    if (r2 > S.cut_g2g2f * 1.00001f) return true;
    const double o[3] = {S.g_cm[3 * h], S.g_cm[3 * h + 1], S.g_cm[3 * h + 2]};
    return sqdist_d(S, cm, o) >= S.cut_g2g2;
}

// quaternion rotation v' = v + w t + u x t, t = 2 u x v (FP64, no contraction)
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

// ---------------------------------------------------------------- proposals
struct Proposal {
    int kind, index;
    double dr[3];
    double quat[4];
    double u;
    bool rotate;
};

// device RNG proposal (batched mode): a deliberate deviation from the reference's
// mt19937 stream.  Uniform direction (Archimedes), |dr| = dp * U(0,1), uniform
// particle/group choice, 53-bit Metropolis uniform.
__device__ Proposal philox_proposal(const DevSys& S, unsigned long long ctr, uint32_t sys_id, uint64_t seed,
                                    double dp, double dprot, bool molecular)
{
    Proposal p;
    const uint32_t k0 = (uint32_t)seed, k1 = (uint32_t)(seed >> 32);
    const U4 c1 = philox({(uint32_t)ctr, (uint32_t)(ctr >> 32), sys_id, 0u}, k0, k1);
    const U4 c2 = philox({(uint32_t)ctr, (uint32_t)(ctr >> 32), sys_id, 1u}, k0, k1);
    const float z = fmaf(2.f, u01_24(c1.y), -1.f) ;
    float s, c;
    sincospif(2.f * u01_24(c1.z), &s, &c);
    const float rxy = sqrtf(fmaxf(0.f, 1.f - z * z));
    const double len = dp * (double)u01_24(c1.w);
    p.dr[0] = (double)(rxy * c) * len;
    p.dr[1] = (double)(rxy * s) * len;
    p.dr[2] = (double)z * len;
    p.u = u01_53(c2.x, c2.y);
    p.rotate = false;
    p.quat[0] = 1.0;
    p.quat[1] = p.quat[2] = p.quat[3] = 0.0;
    if (!molecular) {
        p.kind = FAU_MOVE_ATOMIC;
        const uint32_t n = S.n_atomic > 0 ? (uint32_t)S.n_atomic : (uint32_t)S.n;
        const uint32_t j = __umulhi(c1.x, n);
        p.index = S.n_atomic > 0 ? S.atomic_idx[j] : (int)j;
    }
    else {
        p.kind = FAU_MOVE_MOLECULAR;
        p.index = (int)__umulhi(c1.x, (uint32_t)S.n_groups);
        if (dprot > 0.0) {
            const float az = fmaf(2.f, u01_24(c2.z), -1.f);
            float as, ac;
            sincospif(2.f * u01_24(c2.w), &as, &ac);
            const float axy = sqrtf(fmaxf(0.f, 1.f - az * az));
            const U4 c3 = philox({(uint32_t)ctr, (uint32_t)(ctr >> 32), sys_id, 2u}, k0, k1);
            const double angle = dprot * ((double)u01_24(c3.x) - 0.5);
            const double ha = 0.5 * angle;
            const double sh = sin(ha);
            p.quat[0] = cos(ha);
            p.quat[1] = sh * (double)(axy * ac);
            p.quat[2] = sh * (double)(axy * as);
            p.quat[3] = sh * (double)az;
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
    p.rotate = !(f.quat[0] == 0.0 && f.quat[1] == 0.0 && f.quat[2] == 0.0 && f.quat[3] == 0.0);
    return p;
}

// (xn - xo) / L per axis under minimum image (Chameleon::vdist src/geometry.h:429-458),
// FP64 difference rounded once to FP32: the Ewald phase increment k.(xn - xo) / 2 pi
// of every k-vector follows from it without cancellation.
__device__ __forceinline__ float3 min_image_frac(const DevSys& S, const double* xn, const double* xo)
{
    float g[3];
#pragma unroll
    for (int d = 0; d < 3; d++) {
        double v = __dsub_rn(xn[d], xo[d]);
        if (v > S.half[d]) v = __dsub_rn(v, S.L[d]);
        else if (v < -S.half[d]) v = __dadd_rn(v, S.L[d]);
        g[d] = (float)v * (float)S.inv[d];
    }
    return make_float3(g[0], g[1], g[2]);
}

// Warp 0 turns a proposal into trial positions (FP64, exact) and records.
// AtomicTranslateRotate::translateParticle (src/move.cpp:225-240);
// Group::translate (src/group.cpp:115-123) then Group::rotate about the new
// mass centre (src/group.cpp:110-113, src/geometry.h:613-627).
__device__ void prepare_move(const DevSys& S, MoveShared& ms, const Proposal& p, int lane)
{
    if (lane == 0) {
        ms.kind = p.kind;
        ms.index = p.index;
        ms.u = p.u;
        ms.stop = 0;
    }
    if (p.kind == FAU_MOVE_ATOMIC) {
        if (lane == 0) {
            const int i = p.index;
            double xo[3] = {S.x[i], S.y[i], S.z[i]};
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
                ms.cell_old = S.cell_of[i];
                ms.cell_new = cell_of_pos(S, xn, rn);
            }
        }
    }
    else if (p.kind == FAU_MOVE_MOLECULAR) {
        const int g = p.index;
        const int b = S.g_begin[g];
        const int m = S.g_begin[g + 1] - b;
        // new mass centre (every lane, identical FP64 result)
        double cm[3];
#pragma unroll
        for (int d = 0; d < 3; d++)
            cm[d] = boundary1(__dadd_rn(S.g_cm[3 * g + d], p.dr[d]), S.L[d], S.half[d], S.inv[d]);
        double dM[3] = {0, 0, 0};
        if (lane < m && m <= kMaxGroupAtoms) {
            const int i = b + lane;
            const double xo[3] = {S.x[i], S.y[i], S.z[i]};
            double v[3];
#pragma unroll
            for (int d = 0; d < 3; d++) v[d] = boundary1(__dadd_rn(xo[d], p.dr[d]), S.L[d], S.half[d], S.inv[d]);
            if (p.rotate) {
#pragma unroll
                for (int d = 0; d < 3; d++) v[d] = boundary1(__dsub_rn(v[d], cm[d]), S.L[d], S.half[d], S.inv[d]);
                quat_rotate(p.quat, v);
#pragma unroll
                for (int d = 0; d < 3; d++) v[d] = boundary1(__dadd_rn(v[d], cm[d]), S.L[d], S.half[d], S.inv[d]);
            }
            const uint4 ro = S.rec[i];
            uint4 rn;
            rn.x = to_fixed(v[0], S.fx_scale[0]);
            rn.y = to_fixed(v[1], S.fx_scale[1]);
            rn.z = to_fixed(v[2], S.fx_scale[2]);
            rn.w = ro.w;
            ms.rec_old[lane] = ro;
            ms.rec_new[lane] = rn;
            const double q = S.itype_qd[ro.w >> 24];
            ms.q[lane] = (float)q;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                ms.xn[lane][d] = v[d];
                ms.xo[lane][d] = xo[d];
                dM[d] = __dmul_rn(q, __dsub_rn(v[d], xo[d]));
            }
            ms.g[lane] = min_image_frac(S, v, xo);
        }
        // sum dM over the group's atoms in atom order (lane 0 gathers)
#pragma unroll
        for (int d = 0; d < 3; d++) {
            double acc = 0.0;
            for (int a = 0; a < m && a < 32; a++) acc = __dadd_rn(acc, __shfl_sync(0xffffffffu, dM[d], a));
            dM[d] = acc;
        }
        if (lane == 0) {
            ms.m = m;
            ms.first = b;
            if (m > kMaxGroupAtoms) ms.stop = FAU_ERR_ARG;
#pragma unroll
            for (int d = 0; d < 3; d++) {
                ms.cm_new[d] = cm[d];
                ms.dM[d] = dM[d];
            }
            ms.cmrec_old = S.g_cmrec[g];
            ms.cmrec_new = make_uint4(to_fixed(cm[0], S.fx_scale[0]), to_fixed(cm[1], S.fx_scale[1]),
                                      to_fixed(cm[2], S.fx_scale[2]), 0u);
        }
    }
    else if (lane == 0) {
        ms.m = 0;
        ms.first = -1;
    }
}

// metropolisCriterion (src/montecarlo.cpp:17-34) for a finite or infinite du
// (NaN handled by the caller).  A FP32 exp decides unless the uniform is
// within 1e-4 of the threshold; then the FP64 comparison u <= exp(-du) decides.
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

// ---------------------------------------------------------------- block reduction
template <int NT>
__device__ __forceinline__ void block_reduce(FF& a, FF& b, float& sc, int& flags, FF* ra, FF* rb, float* rs,
                                             int* rf)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        FF ta{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
        FF tb{__shfl_xor_sync(0xffffffffu, b.hi, o), __shfl_xor_sync(0xffffffffu, b.lo, o)};
        a = ff_sum(a, ta);
        b = ff_sum(b, tb);
        sc += __shfl_xor_sync(0xffffffffu, sc, o);
        flags |= __shfl_xor_sync(0xffffffffu, flags, o);
    }
    if (lane == 0) {
        ra[warp] = a;
        rb[warp] = b;
        rs[warp] = sc;
        rf[warp] = flags;
    }
    __syncthreads();
    if (warp == 0) {
        constexpr int NW = NT / 32;
        a = lane < NW ? ra[lane] : FF{0.f, 0.f};
        b = lane < NW ? rb[lane] : FF{0.f, 0.f};
        sc = lane < NW ? rs[lane] : 0.f;
        flags = lane < NW ? rf[lane] : 0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            FF ta{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
            FF tb{__shfl_xor_sync(0xffffffffu, b.hi, o), __shfl_xor_sync(0xffffffffu, b.lo, o)};
            a = ff_sum(a, ta);
            b = ff_sum(b, tb);
            sc += __shfl_xor_sync(0xffffffffu, sc, o);
            flags |= __shfl_xor_sync(0xffffffffu, flags, o);
        }
    }
}

enum : int { F_NEW_INF = 1, F_OLD_INF = 2, F_NEW_NAN = 4, F_OLD_NAN = 8 };

__device__ __forceinline__ void add_pair(FF& acc, int& flags, float un, float uo, bool ni, bool oi, bool nn, bool on)
{
    ff_add(acc, un - uo);
    flags |= (ni ? F_NEW_INF : 0) | (oi ? F_OLD_INF : 0) | (nn ? F_NEW_NAN : 0) | (on ? F_OLD_NAN : 0);
}

// ---------------------------------------------------------------- the chain kernel
template <int NT, bool PHILOX>
__global__ void __launch_bounds__(NT) chain_kernel(ChainArgs A)
{
    DevSys& S = *A.sys[blockIdx.x];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int K = (S.flags & SYS_EWALD) ? S.K : 0;
    float2* Qf = reinterpret_cast<float2*>(smem_raw);
    float2* pend = Qf + K;
    float2* dlt = pend + K;
    float* Af = reinterpret_cast<float*>(dlt + K);
    int* kn = reinterpret_cast<int*>(Af + K);

    __shared__ PairF pt[kMaxITypes * kMaxITypes];
    __shared__ MoveShared ms;
    __shared__ FF red_a[NT / 32], red_b[NT / 32];
    __shared__ float red_s[NT / 32];
    __shared__ int red_f[NT / 32];

    for (int k = tid; k < K; k += NT) {
        const double2 q = S.Q[k];
        Qf[k] = make_float2((float)q.x, (float)q.y);
        pend[k] = make_float2(0.f, 0.f);
        Af[k] = S.Ak[k];
        kn[k] = S.kn[k];
    }
    for (int t = tid; t < S.nt * S.nt; t += NT) pt[t] = S.pair[t];
    __syncthreads();

    const long long nmoves = A.n_moves ? A.n_moves[blockIdx.x] : A.moves;
    const long long poff = A.prop_off ? A.prop_off[blockIdx.x] : 0;
    const uint32_t sys_id = A.sys_ids ? A.sys_ids[blockIdx.x] : blockIdx.x;
    const unsigned long long ctr0 = A.counters ? A.counters[blockIdx.x] + A.counter_base : A.counter_base;
    const int nt = S.nt;
    const bool molecular_sys = A.molecular ? (A.molecular[blockIdx.x] != 0) : false;
    const float rec_pref_f = (float)S.rec_pref;

    unsigned long long n_acc = 0, n_pairs = 0, n_k = 0, n_mv = 0;
    int since_flush = 0;
    double energy = S.energy, sum_du = 0.0;
    double M[3] = {S.M[0], S.M[1], S.M[2]};
    int err = FAU_OK;
    long long consumed = 0; // proposals fully performed (a stop ends after its move's commit)

    for (long long mv = 0; mv < nmoves; mv++) {
        // ---- 1. proposal -> trial positions (warp 0)
        if (warp == 0) {
            Proposal p;
            if (PHILOX) p = philox_proposal(S, ctr0 + (unsigned long long)mv, sys_id, A.seed, A.dp, A.dprot,
                                            molecular_sys);
            else p = load_proposal(A.props[poff + mv]);
            prepare_move(S, ms, p, lane);
        }
        __syncthreads();
        if (ms.stop) {
            err = ms.stop;
            break;
        }
        const int kind = ms.kind;
        const int m = ms.m;

        // ---- 2. energy change of the moved atoms
        FF accp{0.f, 0.f}, accr{0.f, 0.f};
        float scale = 0.f;
        int flags = 0;
        if (kind != FAU_MOVE_NONE) {
            // Ewald reciprocal: dU = C sum_k A_k (2 Re(Q* d) + |d|^2), d = sum_a q_a (e_new - e_old)
            for (int k = tid; k < K; k += NT) {
                int nx, ny, nz;
                kn_unpack(kn[k], nx, ny, nz);
                // d = sum_a q_a (e^{i phi_new} - e^{i phi_old}) = sum_a 2 q_a sin(D/2) i e^{i(phi_old + D/2)},
                // D = k.(r_new - r_old): no cancellation for small moves
                float2 d = make_float2(0.f, 0.f);
                for (int a = 0; a < m; a++) {
                    const float2 eo = eikr32(nx, ny, nz, ms.rec_old[a]);
                    const float3 g = ms.g[a];
                    const float t = fmaf((float)nx, g.x, fmaf((float)ny, g.y, (float)nz * g.z)); // D/2 in units of pi
                    float sh, ch;
                    sincospif(t, &sh, &ch);
                    const float f = 2.f * ms.q[a] * sh;
                    d.x = fmaf(f, fmaf(-eo.x, sh, -eo.y * ch), d.x);
                    d.y = fmaf(f, fmaf(eo.x, ch, -eo.y * sh), d.y);
                }
                dlt[k] = d;
                const float2 qf = Qf[k], pe = pend[k];
                const float qx = qf.x + pe.x, qy = qf.y + pe.y;
                const float cross = 2.f * fmaf(qx, d.x, qy * d.y);
                const float dd = fmaf(d.x, d.x, d.y * d.y);
                ff_add(accr, Af[k] * (cross + dd));
                scale += rec_pref_f * Af[k] * (fabsf(cross) + dd);
            }
            n_k += (unsigned long long)m * ((K - tid + NT - 1) / NT > 0 ? (K - tid + NT - 1) / NT : 0);

            if (kind == FAU_MOVE_ATOMIC) {
                const int i = ms.index;
                const uint4 rn = ms.rec_new[0], ro = ms.rec_old[0];
                const int ti = rn.w >> 24;
                if (S.flags & SYS_CELLS) {
                    const int nbx = S.off_max[0] - S.off_min[0] + 1;
                    const int nby = S.off_max[1] - S.off_min[1] + 1;
                    const int nbz = S.off_max[2] - S.off_min[2] + 1;
                    const int nnb = nbx * nby * nbz;
                    int G = NT / (2 * nnb);
                    if (G < 1) G = 1;
                    const int items = 2 * nnb * G;
                    for (int it = tid; it < items; it += NT) {
                        const int sc = it / G, sub = it - sc * G;
                        const int state = sc / nnb, c = sc - state * nnb;
                        const int center = state ? ms.cell_new : ms.cell_old;
                        int cc[3];
                        cc[0] = center % S.cdim[0];
                        cc[1] = (center / S.cdim[0]) % S.cdim[1];
                        cc[2] = center / (S.cdim[0] * S.cdim[1]);
                        const int o[3] = {c % nbx + S.off_min[0], (c / nbx) % nby + S.off_min[1],
                                          c / (nbx * nby) + S.off_min[2]};
                        int nc[3];
#pragma unroll
                        for (int d = 0; d < 3; d++) {
                            int v = cc[d] + o[d];
                            if (v < 0) v += S.cdim[d];
                            else if (v >= S.cdim[d]) v -= S.cdim[d];
                            nc[d] = v;
                        }
                        const int cell = nc[0] + S.cdim[0] * (nc[1] + S.cdim[1] * nc[2]);
                        const int cnt = S.cell_cnt[cell];
                        const uint4* cr = S.cell_rec + (size_t)cell * S.cap;
                        const uint4 ri = state ? rn : ro;
                        const double* xi = state ? ms.xn[0] : ms.xo[0];
                        for (int s = sub; s < cnt; s += G) {
                            const uint4 rj = cr[s];
                            const int j = (int)(rj.w & 0xFFFFFFu);
                            if (j == i) continue;
                            const int pidx = ti * nt + (rj.w >> 24);
                            const PairF p = pt[pidx];
                            bool inf = false, nan = false;
                            const float u = pair_u32(S, p, pidx, r2_fixed(S, ri, rj), xi, j, inf, nan, scale);
                            if (state) add_pair(accp, flags, u, 0.f, inf, false, nan, false);
                            else add_pair(accp, flags, 0.f, u, false, inf, false, nan);
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
                        bool ni = false, nn = false, oi = false, on = false;
                        const float un = pair_u32(S, p, pidx, r2_fixed(S, rn, rj), ms.xn[0], j, ni, nn, scale);
                        const float uo = pair_u32(S, p, pidx, r2_fixed(S, ro, rj), ms.xo[0], j, oi, on, scale);
                        add_pair(accp, flags, un, uo, ni, oi, nn, on);
                        n_pairs += 2;
                    }
                }
            }
            else { // molecular: group2all(group) with GroupCutoff, internal energy unchanged
                const int g = ms.index;
                const uint4 cmo = ms.cmrec_old, cmn = ms.cmrec_new;
                const double cmo_d[3] = {S.g_cm[3 * g], S.g_cm[3 * g + 1], S.g_cm[3 * g + 2]};
                for (int h = tid; h < S.n_groups; h += NT) {
                    if (h == g || (S.g_flags[h] & FAU_GROUP_ATOMIC)) continue;
                    const bool cut_o = group_cut(S, cmo, cmo_d, h);
                    const bool cut_n = group_cut(S, cmn, ms.cm_new, h);
                    if (cut_o && cut_n) continue;
                    const int hb = S.g_begin[h], he = S.g_begin[h + 1];
                    for (int b = hb; b < he; b++) {
                        const uint4 rb = S.rec[b];
                        const int tb = rb.w >> 24;
                        for (int a = 0; a < m; a++) {
                            const int pidx = (ms.rec_new[a].w >> 24) * nt + tb;
                            const PairF p = pt[pidx];
                            bool ni = false, nn = false, oi = false, on = false;
                            const float un = cut_n ? 0.f
                                                   : pair_u32(S, p, pidx, r2_fixed(S, ms.rec_new[a], rb), ms.xn[a], b,
                                                              ni, nn, scale);
                            const float uo = cut_o ? 0.f
                                                   : pair_u32(S, p, pidx, r2_fixed(S, ms.rec_old[a], rb), ms.xo[a], b,
                                                              oi, on, scale);
                            add_pair(accp, flags, un, uo, ni, oi, nn, on);
                            n_pairs += (cut_n ? 0 : 1) + (cut_o ? 0 : 1);
                        }
                    }
                }
                for (int t = tid; t < S.n_atomic; t += NT) { // atomic groups are never cut
                    const int b = S.atomic_idx[t];
                    const uint4 rb = S.rec[b];
                    const int tb = rb.w >> 24;
                    for (int a = 0; a < m; a++) {
                        const int pidx = (ms.rec_new[a].w >> 24) * nt + tb;
                        const PairF p = pt[pidx];
                        bool ni = false, nn = false, oi = false, on = false;
                        const float un =
                            pair_u32(S, p, pidx, r2_fixed(S, ms.rec_new[a], rb), ms.xn[a], b, ni, nn, scale);
                        const float uo =
                            pair_u32(S, p, pidx, r2_fixed(S, ms.rec_old[a], rb), ms.xo[a], b, oi, on, scale);
                        add_pair(accp, flags, un, uo, ni, oi, nn, on);
                        n_pairs += 2;
                    }
                }
            }
        }

        // ---- 3. reduce, decide (thread 0)
        block_reduce<NT>(accp, accr, scale, flags, red_a, red_b, red_s, red_f);
        if (tid == 0) {
            double du = 0.0;
            int accept = 0;
            if (kind != FAU_MOVE_NONE) {
                const double du_nb = ff_value(accp);
                const double du_rec = K ? S.rec_pref * ff_value(accr) : 0.0;
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
                const double fin = du_nb + (du_rec + du_surf);
                du = energy_change(fin, flags & F_NEW_INF, flags & F_OLD_INF, flags & F_NEW_NAN, flags & F_OLD_NAN);
                const double x = du * S.beta_scale;
                if (A.pending) {
                    // evaluate only: hand the trial to the caller's Metropolis
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
                    err = FAU_ERR_NAN;
                    ms.stop = FAU_ERR_NAN;
                }
                else {
                    accept = metropolis(x, ms.u) ? 1 : 0;
                }
                if (A.detail) {
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
                n_mv++;
            }
            if (A.acc_out) A.acc_out[poff + mv] = (uint8_t)accept;
            if (A.du_out) A.du_out[poff + mv] = du;
            ms.accept = accept;
        }
        __syncthreads();
        if (ms.stop) {
            err = ms.stop;
            break;
        }

        if (A.pending_dq) // evaluate only: the trial's Q(k) change for a later commit
            for (int k = tid; k < K; k += NT) A.pending_dq[k] = make_double2((double)dlt[k].x, (double)dlt[k].y);

        // ---- 4. commit on accept (State::sync trial -> accepted)
        if (ms.accept) {
            for (int k = tid; k < K; k += NT) {
                const float2 d = dlt[k];
                float2 pe = pend[k];
                pe.x += d.x;
                pe.y += d.y;
                pend[k] = pe;
            }
            if (++since_flush == kFlushAccepts) {
                since_flush = 0;
                for (int k = tid; k < K; k += NT) {
                    double2 q = S.Q[k];
                    const float2 pe = pend[k];
                    q.x += (double)pe.x;
                    q.y += (double)pe.y;
                    S.Q[k] = q;
                    Qf[k] = make_float2((float)q.x, (float)q.y);
                    pend[k] = make_float2(0.f, 0.f);
                }
            }
            if (tid < m) {
                const int i = ms.first + tid;
                S.x[i] = ms.xn[tid][0];
                S.y[i] = ms.xn[tid][1];
                S.z[i] = ms.xn[tid][2];
                S.rec[i] = ms.rec_new[tid];
            }
            if (tid == 0) {
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
                        S.cell_cnt[co] = last;
                        const int sn = S.cell_cnt[cn];
                        if (sn >= S.cap) {
                            err = FAU_ERR_CAPACITY;
                            ms.stop = FAU_ERR_CAPACITY;
                            // keep the particle listed in its old cell so the list stays whole
                            S.cell_rec[(size_t)co * S.cap + last] = ms.rec_new[0];
                            S.slot_of[i] = last;
                            S.cell_cnt[co] = last + 1;
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
        }
        __syncthreads();
        consumed = mv + 1;
        if (ms.stop) {
            err = ms.stop;
            break;
        }
    }

    // flush the pending Q deltas into the FP64 master
    for (int k = tid; k < K; k += NT) {
        const float2 pe = pend[k];
        if (pe.x != 0.f || pe.y != 0.f) {
            double2 q = S.Q[k];
            q.x += (double)pe.x;
            q.y += (double)pe.y;
            S.Q[k] = q;
        }
    }
    // statistics
    __shared__ unsigned long long red_u[NT / 32][2];
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
        for (int w = 0; w < NT / 32; w++) {
            pa += red_u[w][0];
            kb += red_u[w][1];
        }
        S.pair_evals += pa;
        S.k_updates += kb;
        S.moves += n_mv;
        S.accepted += n_acc;
        S.sum_du += sum_du;
        S.energy = energy;
#pragma unroll
        for (int d = 0; d < 3; d++) S.M[d] = M[d];
        if (err != FAU_OK) S.err = err;
        S.consumed = consumed;
    }
}

// ---------------------------------------------------------------- FP64 total energy
__device__ __forceinline__ double block_sum_d(double v, double* red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double s = 0.0;
    if (threadIdx.x == 0)
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    __syncthreads();
    return s;
}

// Nonbonded pairing.all: each i pairs with j > i; same group only if not rigid,
// different groups unless the group cutoff applies.  out[0] += finite sum,
// flags[0] |= 1 for +inf terms, 2 for NaN terms.
__global__ void total_pair_kernel(const DevSys* Sp, double* out, int* flags)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0;
    int f = 0;
    const long long n = S.n;
    for (long long i = blockIdx.x; i < n; i += gridDim.x) {
        const double xi[3] = {S.x[i], S.y[i], S.z[i]};
        const int ti = S.rec[i].w >> 24;
        const int gi = S.group_of[i];
        const bool ai = S.g_flags[gi] & FAU_GROUP_ATOMIC;
        const bool rigid_i = S.g_flags[gi] & FAU_GROUP_RIGID;
        const double cmi[3] = {S.g_cm[3 * gi], S.g_cm[3 * gi + 1], S.g_cm[3 * gi + 2]};
        for (long long j = i + 1 + threadIdx.x; j < n; j += blockDim.x) {
            const int gj = S.group_of[j];
            if (gj == gi) {
                if (rigid_i) continue;
            }
            else if (S.cut_g2g2 >= 0.0 && !ai && !(S.g_flags[gj] & FAU_GROUP_ATOMIC)) {
                const double cmj[3] = {S.g_cm[3 * gj], S.g_cm[3 * gj + 1], S.g_cm[3 * gj + 2]};
                if (sqdist_d(S, cmi, cmj) >= S.cut_g2g2) continue;
            }
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const double u = pair_u64(S, ti, S.rec[j].w >> 24, sqdist_d(S, xi, xj));
            if (isnan(u)) f |= 2;
            else if (isinf(u)) f |= 1;
            else e += u;
        }
    }
    const double s = block_sum_d(e, red);
    if (f) atomicOr(flags, f);
    if (threadIdx.x == 0) out[blockIdx.x] = s; // per-block partial: summed in block order on the host
}

// out[2b] = sum_k A_k |Q_k|^2, out[2b+1] = sum_i self(i), per block b
__global__ void total_misc_kernel(const DevSys* Sp, double* out)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0, s = 0.0;
    if (S.flags & SYS_EWALD)
        for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.K; k += gridDim.x * blockDim.x) {
            const double2 q = S.Q[k];
            e += S.Akd[k] * (q.x * q.x + q.y * q.y);
        }
    if (S.flags & SYS_SELF)
        for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < S.n; i += gridDim.x * blockDim.x)
            s += S.itype_self[S.rec[i].w >> 24];
    const double te = block_sum_d(e, red);
    const double ts = block_sum_d(s, red);
    if (threadIdx.x == 0) {
        out[2 * blockIdx.x] = te;
        out[2 * blockIdx.x + 1] = ts;
    }
}

// ---------------------------------------------------------------- FP64 Q(k) rebuild
// Q_k = sum_j q_j e^{i k.r_j} from the FP64 master positions with k = 2 pi n / L
// and k.r = (kx x + ky y) + kz z, as PolicyIonIon::updateComplex
// (src/energy.cpp:191-206).  One CTA per k.
__global__ void q_rebuild_kernel(const DevSys* Sp, double2* out)
{
    const DevSys& S = *Sp;
    __shared__ double rx[32], ry[32];
    const double twopi = 6.283185307179586476925286766559;
    for (int k = blockIdx.x; k < S.K; k += gridDim.x) {
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        const double kx = twopi * ((double)nx / S.L[0]), ky = twopi * ((double)ny / S.L[1]),
                     kz = twopi * ((double)nz / S.L[2]);
        double sx = 0.0, sy = 0.0;
        for (int j = threadIdx.x; j < S.n; j += blockDim.x) {
            const double ph = __dadd_rn(__dadd_rn(__dmul_rn(kx, S.x[j]), __dmul_rn(ky, S.y[j])), __dmul_rn(kz, S.z[j]));
            double s, c;
            sincos(ph, &s, &c);
            const double q = S.itype_qd[S.rec[j].w >> 24];
            sx += q * c;
            sy += q * s;
        }
        const double tx = block_sum_d(sx, rx);
        const double ty = block_sum_d(sy, ry);
        if (threadIdx.x == 0) out[k] = make_double2(tx, ty);
    }
}

// ---------------------------------------------------------------- plain FP64 single move
// du of moving m atoms (new FP64 positions in P.xn), FP64 pair math from the FP64
// master positions (sqdist) and FP64 Ewald phases k.r (src/energy.cpp:219-247).
__global__ void plain_pair_kernel(const DevSys* Sp, const PlainMove* P, double* out, int* flags)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0, sc = 0.0;
    int f = 0;
    const int m = P->m;
    for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < S.n; j += gridDim.x * blockDim.x) {
        const int gj = S.group_of[j];
        if (P->kind == FAU_MOVE_ATOMIC) {
            const int i = P->first;
            if (j == i) continue;
            const int ti = S.rec[i].w >> 24, tj = S.rec[j].w >> 24;
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const double xo[3] = {S.x[i], S.y[i], S.z[i]};
            const double un = pair_u64(S, ti, tj, sqdist_d(S, P->xn[0], xj));
            const double uo = pair_u64(S, ti, tj, sqdist_d(S, xo, xj));
            if (isnan(un)) f |= 4; else if (isinf(un)) f |= 1; else { e += un; sc += fabs(un); }
            if (isnan(uo)) f |= 8; else if (isinf(uo)) f |= 2; else { e -= uo; sc += fabs(uo); }
        }
        else {
            const int g = P->group;
            if (gj == g) continue;
            bool cut_o = false, cut_n = false;
            if (S.cut_g2g2 >= 0.0 && !(S.g_flags[gj] & FAU_GROUP_ATOMIC)) {
                const double cmj[3] = {S.g_cm[3 * gj], S.g_cm[3 * gj + 1], S.g_cm[3 * gj + 2]};
                const double cmo[3] = {S.g_cm[3 * g], S.g_cm[3 * g + 1], S.g_cm[3 * g + 2]};
                cut_o = sqdist_d(S, cmo, cmj) >= S.cut_g2g2;
                cut_n = sqdist_d(S, P->cm_new, cmj) >= S.cut_g2g2;
            }
            const double xj[3] = {S.x[j], S.y[j], S.z[j]};
            const int tj = S.rec[j].w >> 24;
            for (int a = 0; a < m; a++) {
                const int i = P->first + a;
                const int ti = S.rec[i].w >> 24;
                if (!cut_n) {
                    const double un = pair_u64(S, ti, tj, sqdist_d(S, P->xn[a], xj));
                    if (isnan(un)) f |= 4; else if (isinf(un)) f |= 1; else { e += un; sc += fabs(un); }
                }
                if (!cut_o) {
                    const double xo[3] = {S.x[i], S.y[i], S.z[i]};
                    const double uo = pair_u64(S, ti, tj, sqdist_d(S, xo, xj));
                    if (isnan(uo)) f |= 8; else if (isinf(uo)) f |= 2; else { e -= uo; sc += fabs(uo); }
                }
            }
        }
    }
    const double s = block_sum_d(e, red);
    const double s2 = block_sum_d(sc, red);
    if (f) atomicOr(flags, f);
    if (threadIdx.x == 0) {
        atomicAdd(out, s);
        atomicAdd(out + 2, s2);
    }
}

__global__ void plain_ewald_kernel(const DevSys* Sp, const PlainMove* P, double2* dq, double* out)
{
    const DevSys& S = *Sp;
    __shared__ double red[32];
    double e = 0.0;
    const double twopi = 6.283185307179586476925286766559;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.K; k += gridDim.x * blockDim.x) {
        int nx, ny, nz;
        kn_unpack(S.kn[k], nx, ny, nz);
        const double kx = twopi * ((double)nx / S.L[0]), ky = twopi * ((double)ny / S.L[1]),
                     kz = twopi * ((double)nz / S.L[2]);
        double dx = 0.0, dy = 0.0;
        for (int a = 0; a < P->m; a++) {
            const int i = P->first + a;
            const double q = S.itype_qd[S.rec[i].w >> 24];
            const double pn = (kx * P->xn[a][0] + ky * P->xn[a][1]) + kz * P->xn[a][2];
            const double po = (kx * S.x[i] + ky * S.y[i]) + kz * S.z[i];
            double sn, cn, so, co;
            sincos(pn, &sn, &cn);
            sincos(po, &so, &co);
            dx += q * cn - q * co;
            dy += q * sn - q * so;
        }
        dq[k] = make_double2(dx, dy);
        const double2 Q = S.Q[k];
        const double nx2 = (Q.x + dx) * (Q.x + dx) + (Q.y + dy) * (Q.y + dy);
        const double ox2 = Q.x * Q.x + Q.y * Q.y;
        e += S.Akd[k] * (nx2 - ox2);
    }
    const double s = block_sum_d(e, red);
    if (threadIdx.x == 0) atomicAdd(out + 1, s);
}

// commit of a plain move: positions, records, mass centre, cell list, Q += dq
__global__ void plain_commit_kernel(DevSys* Sp, const PlainMove* P, const double2* dq)
{
    DevSys& S = *Sp;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < S.K; k += gridDim.x * blockDim.x) {
        double2 q = S.Q[k];
        q.x += dq[k].x;
        q.y += dq[k].y;
        S.Q[k] = q;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        for (int a = 0; a < P->m; a++) {
            const int i = P->first + a;
            S.x[i] = P->xn[a][0];
            S.y[i] = P->xn[a][1];
            S.z[i] = P->xn[a][2];
            uint4 r = S.rec[i];
            r.x = to_fixed(P->xn[a][0], S.fx_scale[0]);
            r.y = to_fixed(P->xn[a][1], S.fx_scale[1]);
            r.z = to_fixed(P->xn[a][2], S.fx_scale[2]);
            S.rec[i] = r;
            if ((S.flags & SYS_CELLS) && P->kind == FAU_MOVE_ATOMIC) {
                const int co = S.cell_of[i];
                const int cn = cell_of_pos(S, P->xn[a], r);
                const int so = S.slot_of[i];
                if (co == cn) {
                    S.cell_rec[(size_t)co * S.cap + so] = r;
                }
                else {
                    const int last = S.cell_cnt[co] - 1;
                    if (so != last) {
                        const uint4 mvd = S.cell_rec[(size_t)co * S.cap + last];
                        S.cell_rec[(size_t)co * S.cap + so] = mvd;
                        S.slot_of[mvd.w & 0xFFFFFFu] = so;
                    }
                    S.cell_cnt[co] = last;
                    const int sn = S.cell_cnt[cn];
                    if (sn >= S.cap) {
                        S.cell_rec[(size_t)co * S.cap + last] = r;
                        S.slot_of[i] = last;
                        S.cell_cnt[co] = last + 1;
                        S.err = FAU_ERR_CAPACITY;
                    }
                    else {
                        S.cell_rec[(size_t)cn * S.cap + sn] = r;
                        S.cell_cnt[cn] = sn + 1;
                        S.cell_of[i] = cn;
                        S.slot_of[i] = sn;
                    }
                }
            }
        }
        if (P->kind == FAU_MOVE_MOLECULAR) {
            const int g = P->group;
            for (int d = 0; d < 3; d++) S.g_cm[3 * g + d] = P->cm_new[d];
            S.g_cmrec[g] = make_uint4(to_fixed(P->cm_new[0], S.fx_scale[0]), to_fixed(P->cm_new[1], S.fx_scale[1]),
                                      to_fixed(P->cm_new[2], S.fx_scale[2]), 0u);
        }
        for (int d = 0; d < 3; d++) S.M[d] += P->dM[d];
        S.energy += P->du;
        S.moves += P->count_move;
        S.accepted += 1;
        S.sum_du += P->du;
    }
}

// ---------------------------------------------------------------- launchers
size_t chain_smem_bytes(int K) { return (size_t)K * (3 * sizeof(float2) + sizeof(float) + sizeof(int)); }

// dynamic shared memory granted so far per kernel variant (raised on demand,
// never inside a stream capture: the batch runner calls prepare_chain first)
template <int NT, bool PH>
static cudaError_t prepare_chain_t(size_t smem)
{
    static size_t granted = 48 * 1024;
    if (smem <= granted) return cudaSuccess;
    cudaError_t e = cudaFuncSetAttribute(chain_kernel<NT, PH>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) granted = smem;
    return e;
}

template <int NT, bool PH>
static cudaError_t launch_chain_t(const ChainArgs& a, int nblocks, int K, cudaStream_t st)
{
    const size_t smem = chain_smem_bytes(K);
    cudaError_t e = prepare_chain_t<NT, PH>(smem);
    if (e != cudaSuccess) return e;
    chain_kernel<NT, PH><<<nblocks, NT, smem, st>>>(a);
    return cudaGetLastError();
}

cudaError_t prepare_chain(int K, int threads, bool philox)
{
    const size_t smem = chain_smem_bytes(K);
    switch (threads) {
    case 128: return philox ? prepare_chain_t<128, true>(smem) : prepare_chain_t<128, false>(smem);
    case 512: return philox ? prepare_chain_t<512, true>(smem) : prepare_chain_t<512, false>(smem);
    default: return philox ? prepare_chain_t<256, true>(smem) : prepare_chain_t<256, false>(smem);
    }
}

cudaError_t launch_chain(const ChainArgs& a, int nblocks, int K, int threads, bool philox, cudaStream_t st)
{
    switch (threads) {
    case 128:
        return philox ? launch_chain_t<128, true>(a, nblocks, K, st) : launch_chain_t<128, false>(a, nblocks, K, st);
    case 512:
        return philox ? launch_chain_t<512, true>(a, nblocks, K, st) : launch_chain_t<512, false>(a, nblocks, K, st);
    default:
        return philox ? launch_chain_t<256, true>(a, nblocks, K, st) : launch_chain_t<256, false>(a, nblocks, K, st);
    }
}

// Partials layout in d_out: [0, kTotalPairBlocks) pair sums per block, then
// 2 * kTotalMiscBlocks (reciprocal, self) pairs; unused blocks write nothing, so
// the caller zeroes the buffer first.  Deterministic: no floating-point atomics.
cudaError_t launch_total(const DevSys* dsys, int n, int K, double* d_out, int* d_flags, cudaStream_t st)
{
    int blocks = n < kTotalPairBlocks ? (n > 0 ? n : 1) : kTotalPairBlocks;
    total_pair_kernel<<<blocks, 256, 0, st>>>(dsys, d_out, d_flags);
    int kb = (K + n + 255) / 256;
    if (kb < 1) kb = 1;
    if (kb > kTotalMiscBlocks) kb = kTotalMiscBlocks;
    total_misc_kernel<<<kb, 256, 0, st>>>(dsys, d_out + kTotalPairBlocks);
    return cudaGetLastError();
}

cudaError_t launch_q_rebuild(const DevSys* dsys, int K, double2* out, cudaStream_t st)
{
    if (K <= 0) return cudaSuccess;
    q_rebuild_kernel<<<K < 2048 ? K : 2048, 256, 0, st>>>(dsys, out);
    return cudaGetLastError();
}

cudaError_t launch_plain_du(const DevSys* dsys, const PlainMove* pm, int n, int K, double2* dq, double* out, int* flags,
                            cudaStream_t st)
{
    int b = (n + 255) / 256;
    if (b < 1) b = 1;
    if (b > 1024) b = 1024;
    plain_pair_kernel<<<b, 256, 0, st>>>(dsys, pm, out, flags);
    if (K > 0) {
        int kb = (K + 255) / 256;
        plain_ewald_kernel<<<kb, 256, 0, st>>>(dsys, pm, dq, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_plain_commit(DevSys* dsys, const PlainMove* pm, int K, const double2* dq, cudaStream_t st)
{
    int kb = (K + 255) / 256;
    if (kb < 1) kb = 1;
    plain_commit_kernel<<<kb, 256, 0, st>>>(dsys, pm, dq);
    return cudaGetLastError();
}

} // namespace fau
